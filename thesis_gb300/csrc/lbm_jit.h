// Run-time specialisation of the step kernel (lbm_jit.cpp).
#pragma once
#include <cuda_runtime.h>

#include <string>

namespace lbm {

struct JitStepKey {
    int q, coll, storage;
    bool phys, wrap;
    int nx, ny, nz;
    int block;          // threads per block along x
    int hint;           // population load form (ld_pop)
    bool pred;          // blocked links by predicated loads
    bool compile_only;  // compile to a cubin and stop (no GPU needed)
    bool pair;          // two nodes per thread (step_kernel_x2_fixed; hint, pred unused)
    int minb = 1;       // __launch_bounds__ minimum blocks per SM (1: no constraint)
    bool hspace = false;  // one node per thread in storage units (step_kernel_h_fixed)
    int zwalk = 1;        // storage units: nodes a thread updates along z (flag word loaded ahead)
    bool zpair = false;   // storage units, zwalk even: two z nodes at a time on packed FP32x2
};

// Compile (or fetch from the process cache) step_kernel_fixed for `k` and
// return its handle; launch it with cudaLaunchKernel((const void *)kernel,
// ...) and a StepParams argument.  Returns 0 or -1 with `err` set.
int jit_step_kernel(const JitStepKey &k, cudaKernel_t *out, std::string &err);

}  // namespace lbm
