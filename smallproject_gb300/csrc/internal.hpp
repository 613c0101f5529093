// internal.hpp - error reporting shared by the C-ABI translation units.
#pragma once
#include <cstdint>
#include <string>
#include "vxr.h"

namespace vxr {
int set_error(int code, const std::string& msg);   // stores msg for vxr_last_error, returns code
void clear_error();
// "device error flags 0x<hex> (<name of every set bit>)" for a kernel error word:
// 2 temporal light index, 4 spatial light index, 8 shading light index,
// 16 a tensor-core (mbarrier) wait of the proposal inference gave up
std::string device_flags_message(uint32_t flags);
}  // namespace vxr

#define VXR_CHECK_ARG(cond, msg) \
    do {                          \
        if (!(cond)) return ::vxr::set_error(VXR_E_INVALID, msg); \
    } while (0)
