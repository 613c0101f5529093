// internal.hpp - error reporting shared by the C-ABI translation units.
#pragma once
#include <string>
#include "vxr.h"

namespace vxr {
int set_error(int code, const std::string& msg);   // stores msg for vxr_last_error, returns code
void clear_error();
}  // namespace vxr

#define VXR_CHECK_ARG(cond, msg) \
    do {                          \
        if (!(cond)) return ::vxr::set_error(VXR_E_INVALID, msg); \
    } while (0)
