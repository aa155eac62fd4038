"""Builds 2dtissue_gb300/_build/lib2dtissue_gb300.so in-tree.

Host C++ (mesh, chart, tables) with g++ and the CUDA translation unit with nvcc for sm_103a
only; translation units compile in parallel. Host code uses -ffp-contract=off so that the chart
and the placement draws are bit-identical on x86-64 and aarch64.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "lib2dtissue_gb300.so")
CLI = os.path.join(OUT, "tds_cli")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")

HOST_SRCS = ["mesh.cpp", "geometry.cpp"]
CUDA_SRCS = ["capi.cu", "ref_step.cu"]
# ref_step.cu restates the reference's FP64 arithmetic: no multiply-add contraction, so that it
# rounds like the oracle (built with -ffp-contract=off)
CUDA_FLAGS = {"ref_step.cu": ["--fmad=false"]}
HEADERS = ["mesh.hpp", "geometry.hpp", "kernels.cuh", "philox.cuh", "adjoint.cuh"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stderr


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "tds.h")]
    jobs = []
    objs = []
    for src in HOST_SRCS:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-c", s, "-o", o])
    for src in CUDA_SRCS:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            cmd = [NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "--extended-lambda",
                                   "-Xcompiler", "-fPIC,-ffp-contract=off", "-c", s, "-o", o] + CUDA_FLAGS.get(src, [])
            if ptxas_info:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for err in ex.map(_run, jobs):
            if (verbose or ptxas_info) and err:
                sys.stderr.write(err)
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        _run([NVCC] + ARCH + ["-shared", "-o", tmp] + objs)
        os.replace(tmp, LIB)
    cli_src = os.path.join(CSRC, "cli.cpp")
    if force or _stale(CLI, [cli_src, LIB, os.path.join(CSRC, "tissue.hpp")]):
        _run(["g++", "-O2", "-std=c++17", cli_src, "-o", CLI, "-L" + OUT, "-l2dtissue_gb300",
              "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
