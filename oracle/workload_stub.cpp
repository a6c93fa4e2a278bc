// workload_stub.cpp -- the error hook of the workload generator when it is built
// into the oracle's workload library (TEST INFRASTRUCTURE).
//
// oracle/Makefile compiles xvk_ray_gb300/csrc/scene_gen.cpp (the benchmark's
// synthetic scenes and camera UBOs) into _build/libworkload.so, so that the CPU
// baseline generates exactly the scene and camera path the GPU benchmark
// renders without loading libxr.so.  Inside libxr.so, xr::fail also records the
// last-error string; here the status alone is returned.
#include <string>

#include "xr.h"

namespace xr {
struct Context;
xr_status fail(const Context*, xr_status code, const std::string&) { return code; }
}  // namespace xr
