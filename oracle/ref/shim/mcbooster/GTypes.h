// Project-written stand-ins for the MCBooster names the reference's amplitude PDFs use (MCBooster is an
// empty submodule of the reference; nothing here is copied from it).  Scalar types.
#pragma once
#if !defined(__CUDACC__)
#ifndef __host__
#define __host__
#endif
#ifndef __device__
#define __device__
#endif
#endif
namespace mcbooster {
typedef double GReal_t;
typedef int GInt_t;
typedef unsigned int GUInt_t;
typedef long GLong_t;
typedef bool GBool_t;
} // namespace mcbooster
