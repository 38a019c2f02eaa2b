// Project-written stand-ins for MCBooster's functor interfaces: a functor of n particles writing several
// variables (IFunctionArray, as the reference's Dim5 / Dim2 implement) or returning one (IFunction).
#pragma once
#include <mcbooster/GTypes.h>
#include <mcbooster/Vector4R.h>

namespace mcbooster {
struct IFunctionArray {
    GInt_t dim = 0;
    virtual ~IFunctionArray() = default;
    virtual void operator()(const GInt_t n, Vector4R **particles, GReal_t *variables) = 0;
};
struct IFunction {
    virtual ~IFunction() = default;
    virtual GReal_t operator()(const GInt_t n, Vector4R **particles) = 0;
};
} // namespace mcbooster
