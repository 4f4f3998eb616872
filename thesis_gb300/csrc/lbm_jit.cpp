// Run-time specialisation of the step kernel for one lattice.
//
// step_kernel_fixed<...> (lbm_step.cuh) is the fused step with nx, ny, nz
// fixed at compile time.  The library carries the kernel sources as strings
// (generated at build time from thesis_gb300/csrc), compiles the instance a
// handle needs with NVRTC straight to an sm_103a cubin, loads it with the
// runtime's library API and launches it like a built-in kernel.  Instances
// are cached for the life of the process, keyed by their template arguments.
#include <cuda_runtime.h>
#include <nvrtc.h>

#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "lbm_jit.h"
#include "jit_sources.h"  // generated: kJitHeaders[], kJitHeaderNames[], kJitHeaderCount

namespace lbm {

namespace {
std::mutex g_jit_mutex;
std::map<std::string, cudaKernel_t> g_jit_cache;

const char *kStdint =
    "#pragma once\n"
    "typedef signed char int8_t; typedef unsigned char uint8_t;\n"
    "typedef short int16_t; typedef unsigned short uint16_t;\n"
    "typedef int int32_t; typedef unsigned int uint32_t;\n"
    "typedef long long int64_t; typedef unsigned long long uint64_t;\n";
const char *kStddef = "#pragma once\ntypedef unsigned long size_t;\n";
}  // namespace

int jit_step_kernel(const JitStepKey &k, cudaKernel_t *out, std::string &err) {
    const std::string common = std::to_string(k.q) + ", " + std::to_string(k.coll) + ", " +
                               std::to_string(k.storage) + ", " + (k.phys ? "true" : "false") + ", " +
                               (k.wrap ? "true" : "false") + ", " + std::to_string(k.nx) + ", " +
                               std::to_string(k.ny) + ", " + std::to_string(k.nz) + ", " + std::to_string(k.block);
    const std::string minb = std::to_string(k.minb > 0 ? k.minb : 1);
    const std::string expr =
        k.pair     ? "lbm::step_kernel_x2_fixed<" + common + ", " + minb + ">"
        : k.hspace ? "lbm::step_kernel_h_fixed<" + common + ", " + minb + (k.pred ? ", true" : ", false") + ", " +
                         std::to_string(k.zwalk > 1 ? k.zwalk : 1) + ", " + std::to_string(k.hint & 1) +
                         (k.zpair && k.zwalk > 1 ? ", true" : ", false") + ">"
                   : "lbm::step_kernel_fixed<" + common + ", " + std::to_string(k.hint) + ", " +
                         (k.pred ? "true" : "false") + ", " + minb + ">";
    {
        std::lock_guard<std::mutex> lock(g_jit_mutex);
        auto it = g_jit_cache.find(expr);
        if (it != g_jit_cache.end() && !k.compile_only) {
            *out = it->second;
            return 0;
        }
    }
    // compile outside the lock: independent programs build in parallel
    std::vector<const char *> hdr, names;
    for (int i = 0; i < kJitHeaderCount; ++i) {
        hdr.push_back(kJitHeaders[i]);
        names.push_back(kJitHeaderNames[i]);
    }
    hdr.push_back(kStdint);
    names.push_back("stdint.h");
    hdr.push_back(kStddef);
    names.push_back("stddef.h");
    const char *src = "#include \"lbm_step_x2.cuh\"\n";
    nvrtcProgram prog;
    nvrtcResult r = nvrtcCreateProgram(&prog, src, "lbm_step_fixed.cu", (int)hdr.size(), hdr.data(), names.data());
    if (r != NVRTC_SUCCESS) {
        err = std::string("nvrtcCreateProgram: ") + nvrtcGetErrorString(r);
        return -1;
    }
    nvrtcAddNameExpression(prog, expr.c_str());
    // cuda_fp16.h comes from the toolkit the library was built against
    const std::string inc = std::string("-I") + THESIS_CUDA_INCLUDE;
    const char *opts[] = {"--gpu-architecture=sm_103a", "-std=c++17", "-lineinfo", inc.c_str()};
    r = nvrtcCompileProgram(prog, 4, opts);
    if (r != NVRTC_SUCCESS) {
        size_t n = 0;
        nvrtcGetProgramLogSize(prog, &n);
        std::string log(n, '\0');
        if (n) nvrtcGetProgramLog(prog, &log[0]);
        err = std::string("nvrtcCompileProgram: ") + nvrtcGetErrorString(r) + "\n" + log;
        nvrtcDestroyProgram(&prog);
        return -1;
    }
    const char *lowered = nullptr;
    nvrtcGetLoweredName(prog, expr.c_str(), &lowered);
    const std::string name = lowered ? lowered : "";
    size_t cubin_size = 0;
    nvrtcGetCUBINSize(prog, &cubin_size);
    std::vector<char> cubin(cubin_size);
    r = nvrtcGetCUBIN(prog, cubin.data());
    nvrtcDestroyProgram(&prog);
    if (r != NVRTC_SUCCESS || name.empty()) {
        err = "nvrtc: no cubin or kernel name for " + expr;
        return -1;
    }
    if (k.compile_only) {
        if (out) *out = nullptr;
        return 0;
    }
    cudaLibrary_t lib;
    cudaError_t e = cudaLibraryLoadData(&lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (e != cudaSuccess) {
        err = std::string("cudaLibraryLoadData: ") + cudaGetErrorString(e);
        return -1;
    }
    cudaKernel_t kern;
    e = cudaLibraryGetKernel(&kern, lib, name.c_str());
    if (e != cudaSuccess) {
        err = std::string("cudaLibraryGetKernel: ") + cudaGetErrorString(e);
        return -1;
    }
    std::lock_guard<std::mutex> lock(g_jit_mutex);
    auto ins = g_jit_cache.emplace(expr, kern);  // another thread may have won
    *out = ins.first->second;
    return 0;
}

}  // namespace lbm
