/* Logging stub for compiling the reference's test driver as a library (TEST INFRASTRUCTURE ONLY,
 * used by oracle/build_ref_cpu.sh): every spdlog macro expands to nothing.  The real header pulls
 * in these standard headers, which the driver relies on. */
#pragma once
#include <algorithm>
#include <limits>
#include <map>
#include <memory>
#include <numeric>
#include <set>
#include <string>
#define SPDLOG_INFO(...) ((void)0)
#define SPDLOG_WARN(...) ((void)0)
#define SPDLOG_ERROR(...) ((void)0)
#define SPDLOG_DEBUG(...) ((void)0)
