/* googletest stub for compiling the reference's test driver as a library (TEST INFRASTRUCTURE
 * ONLY, used by oracle/build_ref_cpu.sh): a TEST body becomes a function that is never called. */
#pragma once
#define TEST(suite, name) void pg_unused_##suite##_##name()
