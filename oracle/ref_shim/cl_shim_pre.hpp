/* cl_shim_pre.hpp — ORACLE test infrastructure: standard headers that must be
 * included before the OpenCL qualifier macros of cl_shim_body.hpp exist. */
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>
#include "../../include/rt_cuda.h"
