// NVRTC wrapper: compile generated CUDA C++ to a cubin for sm_103a.
#include "rtc.h"

#include <nvrtc.h>

#include <cstdint>
#include <cstdio>
#include <unistd.h>
#include <cstdlib>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <sys/stat.h>

namespace gf {

namespace {

std::mutex g_mu;
std::map<std::string, std::vector<char>> g_mem;

// FNV-1a 64-bit
uint64_t fnv1a(const std::string &s) {
    uint64_t h = 1469598103934665603ull;
    for(unsigned char c : s) {
        h ^= c;
        h *= 1099511628211ull;
    }
    return h;
}

std::string cacheDir() {
    const char *d = std::getenv("GF_CACHE_DIR");
    if(d && *d)
        return d;
    const char *home = std::getenv("HOME");
    return std::string(home && *home ? home : "/tmp") + "/.cache/gfengine";
}

void mkdirs(const std::string &p) {
    std::string cur;
    std::stringstream ss(p);
    std::string part;
    if(!p.empty() && p[0] == '/')
        cur = "/";
    while(std::getline(ss, part, '/')) {
        if(part.empty())
            continue;
        cur += part + "/";
        mkdir(cur.c_str(), 0755);
    }
}

} // namespace

std::string rtc_version() {
    int ma = 0, mi = 0;
    nvrtcVersion(&ma, &mi);
    return std::to_string(ma) + "." + std::to_string(mi);
}

bool rtc_compile(const std::string &source, const std::string &arch, std::vector<char> &cubin, std::string &log) {
    const std::string key = arch + "|" + rtc_version() + "|" + source;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        auto it = g_mem.find(key);
        if(it != g_mem.end()) {
            cubin = it->second;
            return true;
        }
    }
    char name[32];
    std::snprintf(name, sizeof name, "%016llx", (unsigned long long)fnv1a(key));
    const bool useDisk = !std::getenv("GF_NO_DISK_CACHE");
    const std::string dir  = cacheDir();
    const std::string path = dir + "/" + name + ".cubin";
    if(useDisk) {
        std::ifstream f(path, std::ios::binary);
        if(f) {
            std::vector<char> buf((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
            if(!buf.empty()) {
                cubin = buf;
                std::lock_guard<std::mutex> lk(g_mu);
                g_mem[key] = buf;
                return true;
            }
        }
    }
    nvrtcProgram prog;
    if(nvrtcCreateProgram(&prog, source.c_str(), "gf_tree.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS) {
        log = "nvrtcCreateProgram failed";
        return false;
    }
    std::string archOpt = "--gpu-architecture=" + arch;
    const char *opts[]  = {archOpt.c_str(), "--std=c++17", "-default-device", "-lineinfo", "--extra-device-vectorization"};
    nvrtcResult r       = nvrtcCompileProgram(prog, 5, opts);
    size_t logSize      = 0;
    nvrtcGetProgramLogSize(prog, &logSize);
    std::string plog(logSize, '\0');
    if(logSize)
        nvrtcGetProgramLog(prog, &plog[0]);
    if(r != NVRTC_SUCCESS) {
        log = std::string("NVRTC: ") + nvrtcGetErrorString(r) + "\n" + plog;
        nvrtcDestroyProgram(&prog);
        return false;
    }
    size_t n = 0;
    if(nvrtcGetCUBINSize(prog, &n) != NVRTC_SUCCESS || n == 0) {
        log = "NVRTC produced no cubin";
        nvrtcDestroyProgram(&prog);
        return false;
    }
    cubin.resize(n);
    nvrtcGetCUBIN(prog, cubin.data());
    nvrtcDestroyProgram(&prog);
    {
        std::lock_guard<std::mutex> lk(g_mu);
        g_mem[key] = cubin;
    }
    if(useDisk) {
        mkdirs(dir);
        std::string tmp = path + ".tmp" + std::to_string((long)getpid());
        std::ofstream f(tmp, std::ios::binary);
        if(f) {
            f.write(cubin.data(), (std::streamsize)cubin.size());
            f.close();
            std::rename(tmp.c_str(), path.c_str());
        }
    }
    return true;
}

} // namespace gf
