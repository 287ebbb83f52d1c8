// Helpers shared by the C-ABI translation units (capi.cpp, batch.cpp).
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "passes.h"
#include "plan.h"

namespace eithot {
namespace api {

// Records `msg` as the calling thread's last error and returns `code`.
int fail(int code, const std::string& msg);

bool elem_ok(size_t e);

// Scratch for a pass list: at least one staged item of every pass, at most
// what lets each pass run as a single group, capped at alpha * bytes when
// that cap still covers the minimum.
size_t choose_workspace(const std::vector<Pass>& passes, const DeviceCaps& caps, double alpha, double bytes);

// Capabilities of the current device.
int device_caps(DeviceCaps* caps);

// Plans and lowers one request.
int build(int rank, const int64_t* dims, const int* perm, size_t elem, int nb, double alpha, int order,
          const DeviceCaps& caps, NdPlan* plan, std::vector<Pass>* passes);

}  // namespace api
}  // namespace eithot
