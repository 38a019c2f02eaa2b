// Project-written stand-in for the CMake-generated version header of the reference (Version.h.in).
#pragma once
#define GOOFIT_VERSION_MAJOR 2
#define GOOFIT_VERSION_MINOR 3
#define GOOFIT_VERSION_PATCH 0
#define GOOFIT_VERSION "2.3.0"
#define GOOFIT_TAG "CPU restatement build (Thrust OMP)"
#define GOOFIT_SOURCE_DIR ""
