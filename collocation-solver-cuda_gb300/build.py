"""Build of the native library libcs_gb300.so (host runtime + C ABI) with nvcc
for sm_103a, in tree, and a compile check of the solver kernels.

The solver kernels themselves are specialised per problem and compiled at run
time by NVRTC (csrc/cs_runtime.cu); `check_kernels` compiles them here with
nvcc for one problem so that a broken kernel fails the build, and reports
registers, spills and shared memory (-Xptxas -v).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcs_gb300.so")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _kernels_header():
    """cs_umma.cuh + cs_kernels.cuh as a C string constant (the NVRTC program
    text after the problem-specific prelude)."""
    os.makedirs(BUILD, exist_ok=True)
    src = open(os.path.join(CSRC, "cs_umma.cuh")).read() + "\n" + open(os.path.join(CSRC, "cs_kernels.cuh")).read()
    out = os.path.join(BUILD, "cs_kernels_src.h")
    delim = "CSKSRC"
    assert (")" + delim + '"') not in src
    text = "// generated from cs_umma.cuh and cs_kernels.cuh by build.py\n"
    # split into chunks: some compilers limit the length of one string literal
    chunks = [src[i:i + 16000] for i in range(0, len(src), 16000)]
    text += "static const char cs_kernels_source[] =\n"
    for c in chunks:
        text += 'R"%s(%s)%s"\n' % (delim, c, delim)
    text += ";\n"
    if not os.path.exists(out) or open(out).read() != text:
        with open(out, "w") as f:
            f.write(text)
    return out


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(force=False, verbose=False):
    hdr = _kernels_header()
    sources = [os.path.join(CSRC, "cs_runtime.cu"), os.path.join(CSRC, "cs_babd.cu"), os.path.join(CSRC, "cs_mlp.cu"),
               os.path.join(CSRC, "cs_tc.cu"), os.path.join(CSRC, "cs_text.cu")]
    deps = sources + [os.path.join(CSRC, "cs_kernels.cuh"), os.path.join(CSRC, "cs_umma.cuh"),
                      os.path.join(CSRC, "cs_dtoa.h"), os.path.join(CSRC, "cs_text.h"),
                      os.path.join(ROOT, "include", "cs_gb300.h"), hdr]
    if not force and not _stale(LIB, deps):
        return LIB
    cmd = [NVCC, "-O3", "-std=c++17", "-lineinfo", *ARCH, "-shared", "-Xcompiler", "-fPIC",
           "-I", os.path.join(ROOT, "include"), "-I", BUILD, "-I", CSRC,
           *sources, "-o", LIB + ".tmp",
           "-L", os.path.join(CUDA_HOME, "lib64"), "-L", os.path.join(CUDA_HOME, "lib64", "stubs"),
           "-lnvrtc"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


def check_kernels(problem_name="vdp", m=4, verbose=False, big=False):
    """nvcc-compile the kernel program for one problem to a cubin and return
    the -Xptxas -v report (big: the large-system kernels)."""
    from . import module as _module  # noqa: F401  (package import)
    from .module import kernel_program_text
    from .ocp import Problem
    pr = Problem.from_file(os.path.join(HERE, "problems", problem_name + ".ocp"))
    text = kernel_program_text(pr, m, big=big)
    os.makedirs(BUILD, exist_ok=True)
    cu = os.path.join(BUILD, "check_%s_m%d%s.cu" % (problem_name, m, "_big" if big else ""))
    with open(cu, "w") as f:
        f.write(text)
    cmd = [NVCC, "-cubin", "-O3", "-std=c++17", "-lineinfo", "-arch=sm_103a", "-Xptxas", "-v", cu,
           "-o", cu[:-3] + ".cubin"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("kernel compile failed:\n" + p.stderr[-6000:])
    if verbose:
        print(p.stderr)
    return p.stderr


if __name__ == "__main__":
    build_library(force="--force" in sys.argv, verbose=True)
