// Project-written stand-in for the CMake-generated header of the reference (Backtrace.h.in): no backtrace
// library in this build.
#pragma once
#define Backtrace_FOUND 0
