// Project-written stand-in for MCBooster's accept-reject flag functor (weight w accepted when
// w > wmax * u for a uniform u drawn from the event index and a seed).
#pragma once
#include <mcbooster/GTypes.h>
#include <thrust/random.h>

namespace mcbooster {
struct FlagAcceptReject {
    GReal_t wmax;
    GInt_t seed;
    FlagAcceptReject(GReal_t w, GInt_t s = 0) : wmax(w), seed(s) {}
    __host__ __device__ GBool_t operator()(GLong_t idx, GReal_t w) const {
        thrust::default_random_engine rng(seed);
        rng.discard(idx);
        thrust::uniform_real_distribution<GReal_t> u(0.0, 1.0);
        return w > wmax * u(rng);
    }
};
} // namespace mcbooster
