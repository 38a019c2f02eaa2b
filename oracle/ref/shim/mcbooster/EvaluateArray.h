// Project-written stand-in for MCBooster's EvaluateArray: applies an IFunctionArray functor to every event
// (one particle of each set per event) and stores its variables in the variable set, event by event.
#pragma once
#include <mcbooster/GContainers.h>
#include <mcbooster/GFunctional.h>

namespace mcbooster {
template <typename FUNCTOR, typename PSET, typename VSET>
void EvaluateArray(FUNCTOR funcObj, PSET &pset, VSET &varset) {
    const size_t np = pset.size(), nv = varset.size();
    const size_t n  = np ? pset[0]->size() : 0;
    std::vector<Vector4R> parts(np);
    std::vector<Vector4R *> ptrs(np);
    std::vector<GReal_t> vars(nv);
    for(size_t i = 0; i < n; ++i) {
        for(size_t k = 0; k < np; ++k) {
            parts[k] = (*pset[k])[i];
            ptrs[k]  = &parts[k];
        }
        funcObj((GInt_t)np, ptrs.data(), vars.data());
        for(size_t j = 0; j < nv; ++j)
            (*varset[j])[i] = vars[j];
    }
}
} // namespace mcbooster
