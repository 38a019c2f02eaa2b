// Project-written: the two functor base classes the reference's functors derive from
// (thrust::unary_function / thrust::binary_function), which the CCCL 3 Thrust in this CUDA toolkit no longer
// provides.  Force-included before every reference source of the CPU build, with <iomanip>, which one
// reference source (Amp3Body_TD.cu) uses without including it.
#pragma once
#include <iomanip>
namespace thrust {
template <typename Arg, typename Result>
struct unary_function {
    using argument_type = Arg;
    using result_type   = Result;
};
template <typename Arg1, typename Arg2, typename Result>
struct binary_function {
    using first_argument_type  = Arg1;
    using second_argument_type = Arg2;
    using result_type          = Result;
};
} // namespace thrust
