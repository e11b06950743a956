// Build configuration of the GB300 TTG runtime (the reference generates ttg/config.h from CMake).
#pragma once
#define TTG_HAVE_COROUTINE 1
#define TTG_HAVE_DEVICE 1
#define TTG_HAVE_CUDA 1
#define TTG_HAVE_CUDART 1
#define TTG_IMPL_DEVICE_SUPPORT 1
