// Run-time compilation of generated kernel sources for sm_103a (NVRTC) and
// loading of the resulting cubin through the CUDA runtime library API.
#pragma once

#include <string>
#include <vector>

namespace gf {

// Compiles `source` to a cubin for the given architecture ("sm_103a").
// Results are cached in memory (per process) and on disk under
// $GF_CACHE_DIR (default ~/.cache/gfengine) keyed by a hash of the source.
// Returns false and sets `log` on failure.
bool rtc_compile(const std::string &source, const std::string &arch, std::vector<char> &cubin, std::string &log);

// Name of the NVRTC version used, e.g. "13.0".
std::string rtc_version();

} // namespace gf
