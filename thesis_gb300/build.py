"""Build recipe for the native library (sm_103a CUDA kernels + C ABI).

Compiles thesis_gb300/csrc/*.cu and *.cpp with nvcc for sm_103a only, in
parallel, into thesis_gb300/_lib/libthesis_lbm.so.  Objects are rebuilt only
when a source or header is newer than the library.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIBNAME = "libthesis_lbm.so"
LIB_PATH = os.path.join(LIBDIR, LIBNAME)
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cand = os.path.join(home, "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def cuda_include():
    """Toolkit include directory (cuda_fp16.h for the run-time kernel build)."""
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    path = os.path.join(home, "include")
    if not os.path.exists(os.path.join(path, "cuda_fp16.h")):
        path = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc()))), "include")
    return path


CLI_DIR = os.path.join(CSRC, "cli")
TOOLS = {"latticegen": "latticegen_main.cpp", "thesis_lbm_run": "lbm_run_main.cpp"}


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def tool_path(name):
    return os.path.join(LIBDIR, name)


def _newest_input():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if os.path.isfile(os.path.join(CSRC, f))]
    files += [os.path.join(CLI_DIR, f) for f in os.listdir(CLI_DIR)]
    inc = os.path.join(ROOT, "include")
    files += [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith(".h")]
    files.append(os.path.abspath(__file__))
    return max(os.path.getmtime(f) for f in files)


# Headers the run-time specialised step kernel is compiled from (lbm_jit.cpp).
JIT_HEADERS = [os.path.join(ROOT, "include", "thesis_lbm.h")] + [
    os.path.join(CSRC, f) for f in ("lbm_types.h", "lbm_device.cuh", "lbm_bc.cuh", "lbm_step.cuh",
                                    "lbm_step_x2.cuh")]


def write_jit_sources(path):
    """Embed the kernel headers as C++ raw strings for NVRTC."""
    delim = "LBMSRC"
    parts, names = [], []
    for h in JIT_HEADERS:
        text = open(h).read()
        if ")" + delim + '"' in text:
            raise RuntimeError("raw-string delimiter found in " + h)
        parts.append('R"%s(%s)%s"' % (delim, text, delim))
        names.append('"%s"' % os.path.basename(h))
    out = ["// generated by thesis_gb300/build.py: kernel headers for NVRTC",
           "#pragma once",
           "static const char *const kJitHeaders[] = {" + ",\n".join(parts) + "};",
           "static const char *const kJitHeaderNames[] = {" + ", ".join(names) + "};",
           "static const int kJitHeaderCount = %d;" % len(names)]
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        f.write("\n".join(out) + "\n")
    os.replace(tmp, path)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def build(force=False, verbose=False):
    """Compile the library if needed; return its path."""
    newest = _newest_input()
    if not force and all(os.path.exists(p) and os.path.getmtime(p) >= newest
                         for p in [LIB_PATH] + [tool_path(t) for t in TOOLS]):
        return LIB_PATH
    os.makedirs(OBJDIR, exist_ok=True)
    write_jit_sources(os.path.join(OBJDIR, "jit_sources.h"))
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2",
              "-I" + os.path.join(ROOT, "include"), "-I" + CSRC, "-I" + OBJDIR,
              '-DTHESIS_CUDA_INCLUDE="%s"' % cuda_include()] + ARCH

    def compile_one(src):
        obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
        cmd = [nvcc()] + common + ["-c", src, "-o", obj]
        if src.endswith(".cpp"):
            # host code: no floating-point contraction, so geometric tests and
            # the generator's comparisons give the same results on every host
            cmd = [nvcc(), "-x", "c++"] + common + ["-Xcompiler", "-ffp-contract=off", "-c", src, "-o", obj]
        out = _run(cmd)
        if verbose and out:
            sys.stdout.write(out)
        return obj

    srcs = sources()
    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB_PATH + ".tmp"
    cuda_lib = os.path.join(os.path.dirname(os.path.dirname(nvcc())), "lib64")
    _run([nvcc(), "-shared"] + ARCH + ["-o", tmp] + objs +
         ["-lcudart", "-lnvrtc", "-Xlinker", "-rpath," + cuda_lib])
    os.replace(tmp, LIB_PATH)
    for name, src in TOOLS.items():
        out = tool_path(name)
        _run(["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), os.path.join(CLI_DIR, src),
              "-o", out + ".tmp",
              "-L" + LIBDIR, "-lthesis_lbm", "-Wl,-rpath,$ORIGIN"])
        os.replace(out + ".tmp", out)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
