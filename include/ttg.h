// TTG API for the GB300 (sm_103a) single-GPU runtime: the subset the device-task path of the
// tiled Cholesky uses (examples/potrf of the reference) — keys, edges, terminals, make_tt,
// send/broadcast, Buffer/devicescratch/TTValue, device::Task coroutines, make_graph_executable,
// execute, fence — with the reference's names and argument meanings.
#pragma once
#include "ttg/runtime.h"
#include "ttg/buffer.h"
#include "ttg/util/multiindex.h"
#include "ttg/tt.h"
#include "ttg/device/task.h"

#define TTG_HAVE_COROUTINE 1
#define TTG_HAVE_DEVICE 1
#define TTG_HAVE_CUDA 1
#define TTG_HAVE_CUDART 1
#define TTG_IMPL_DEVICE_SUPPORT 1
