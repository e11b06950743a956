// ttg::device::Device, current_device(), current_stream(), num_devices() (ttg/ttg/device/device.h).
#pragma once
#include "ttg/runtime.h"
