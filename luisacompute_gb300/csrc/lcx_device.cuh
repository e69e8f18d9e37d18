// The device-side layouts and arithmetic live in the public header, which
// user kernels that call lcx::ray_query (include/lcx/ray_query.cuh) share.
#pragma once
#include "lcx/bvh_device.cuh"
