// The GB300 library's device task queue (gbx_taskq_*, include/gbx_potrf.h) behind the TTG runtime's
// device tasks: after ttg::device::use_gbx_queue(), the tile kernels that device task bodies call on
// ttg::device::current_stream() are recorded into the queue, and the runtime runs each batch as one
// persistent launch (see ttg::rt::DeviceQueue). Unchanged bodies, one launch per batch instead of one
// launch and one host callback per task. Link the application with libgbx_potrf.so.
#pragma once
#include <memory>
#include <stdexcept>
#include <string>

#include "gbx_potrf.h"
#include "ttg/runtime.h"

namespace ttg::device {

class GbxQueue : public rt::DeviceQueue {
  void* q_ = nullptr;

  static void check_status(int st, const char* what) {
    if (st != GBX_OK) throw std::runtime_error(std::string("ttg: ") + what + " failed with status " + std::to_string(st));
  }

 public:
  GbxQueue() { check_status(gbx_taskq_create(&q_), "gbx_taskq_create"); }
  ~GbxQueue() override { gbx_taskq_destroy(q_); }
  GbxQueue(const GbxQueue&) = delete;
  GbxQueue& operator=(const GbxQueue&) = delete;
  cudaStream_t record_stream() override { return static_cast<cudaStream_t>(gbx_taskq_stream(q_)); }
  long long pending() override { return gbx_taskq_pending(q_); }
  void run(cudaStream_t s) override { check_status(gbx_taskq_run(q_, s), "gbx_taskq_run"); }
  void check(cudaStream_t s) override { check_status(gbx_taskq_status(q_, s), "device task queue run"); }
};

/// Routes the device tasks of later executions through a GB300 device task queue (true) or back to
/// one launch per task (false). Call between executions.
inline void use_gbx_queue(bool on = true) {
  rt::Runtime::get().set_device_queue(on ? std::make_shared<GbxQueue>() : nullptr);
}

}  // namespace ttg::device
