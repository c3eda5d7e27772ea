"""Builds libnerfgb.so in-tree with nvcc for sm_103a (no cmake, no torch build
machinery), and its bounds-check build libnerfgb_bounds.so. The translation
units compile in parallel, then link into shared libraries next to this
file.

    python nerf-tf2_gb300/build.py [--force] [--verbose]
"""
import os
import pathlib
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parent
CSRC = HERE / "csrc"
INCLUDE = ROOT / "include"
BUILD = HERE / "_build"
LIB = HERE / "libnerfgb.so"
SOURCES = ["ray_ops.cu", "mlp.cu", "mlp_tc.cu", "gemm_tc.cu", "render.cu", "render_noalloc.cu", "train.cu",
           "proposal.cu", "mlp_train.cu", "mlp_train_bf16.cu", "gate.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build libnerfgb.so")
    return exe


def _flags(extra=()):
    return [*ARCH, "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
            "-Xcompiler", "-fPIC", f"-I{INCLUDE}", f"-I{CSRC}", *extra]


def _stale(target, deps):
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


# Build variants: the library, and the bounds-check build of the same sources
# (every data-dependent index checked, csrc/common.cuh) for the tests.
VARIANTS = {
    "default": (BUILD, LIB, ()),
    "bounds": (HERE / "_build_bounds", HERE / "libnerfgb_bounds.so", ("-DNERF_BOUNDS_CHECK",)),
}


def _plan(variant, force, verbose, extra_flags):
    build_dir, lib, flags = VARIANTS[variant]
    build_dir.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    objs, jobs = [], []
    for src in SOURCES:
        s = CSRC / src
        o = build_dir / (s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s, *headers, pathlib.Path(__file__)]):
            cmd = [nvcc(), *_flags((*flags, *extra_flags)), "-c", str(s), "-o", str(o)]
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    return lib, objs, jobs


def build(force=False, verbose=False, extra_flags=(), variants=("default", "bounds")):
    """Compiles the translation units of every variant in parallel and links
    each library; returns the default library's path."""
    plans = [_plan(v, force, verbose, extra_flags) for v in variants]
    jobs = [j for _, _, js in plans for j in js]

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or r.returncode != 0:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {cmd[-3]}")
    for lib, objs, js in plans:
        if force or js or _stale(lib, objs):
            cmd = [nvcc(), *ARCH, "-shared", "-o", str(lib), *map(str, objs)]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="--verbose" in sys.argv)
    print(LIB)
