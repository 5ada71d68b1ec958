// Library-internal declarations shared by the host-side sources (not part of
// the C ABI).
#pragma once

#include "../../include/fame_gpu.h"

// Records msg as the context's last error and returns code.
int fame_gpu_fail(fame_gpu* g, int code, const char* msg);
// The device of the context.
int fame_gpu_device_of(const fame_gpu* g);
