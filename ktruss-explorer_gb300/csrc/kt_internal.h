// Internal declarations shared by the host and device translation units of libktruss_gb300.
#pragma once

#include "ktruss_gb300.h"

#include <cstdint>
#include <cstdio>
#include <string>

namespace kt {

// Records a formatted message as the thread's last error and returns `code`.
int fail(int code, const char* fmt, ...);
void clear_error();

}  // namespace kt
