// Project-written stand-in for MCBooster's Evaluate (one value per event of an IFunction functor).
#pragma once
#include <mcbooster/EvaluateArray.h>

namespace mcbooster {
template <typename FUNCTOR, typename PSET, typename VEC>
void Evaluate(FUNCTOR funcObj, PSET &pset, VEC &out) {
    const size_t np = pset.size();
    const size_t n  = np ? pset[0]->size() : 0;
    std::vector<Vector4R> parts(np);
    std::vector<Vector4R *> ptrs(np);
    for(size_t i = 0; i < n; ++i) {
        for(size_t k = 0; k < np; ++k) {
            parts[k] = (*pset[k])[i];
            ptrs[k]  = &parts[k];
        }
        out[i] = funcObj((GInt_t)np, ptrs.data());
    }
}
} // namespace mcbooster
