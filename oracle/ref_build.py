"""Build recipe for the reference-kernel harness -- TEST INFRASTRUCTURE.

* PTX of the reference's own kernels, compiled from the reference sources
  (CosmosCuda.cuh) through oracle/ref_kernels.cu, one file per (N, dt) because
  the reference fixes both at compile time.  Built only where the reference
  tree is present; the PTX (text) lands in oracle/_ref/ (git-ignored) and
  travels with the working tree to the GPU machine, which JIT-compiles it.
  Flags follow the reference's build: -O3 --use_fast_math
  (CosmosSimulationWithCuda.vcxproj); target compute_103a.
* oracle/_ref/libref_runner.so from oracle/ref_runner.cpp (host C++ against
  the CUDA driver/runtime and cuFFT), built wherever nvcc is available.

The location of the reference tree comes from the environment
(COSMOS_REFERENCE_ROOT); `make -C oracle ref` sets it to the tree's place in
the build container.  Without it only the runner is built.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REFERENCE_ROOT = os.environ.get("COSMOS_REFERENCE_ROOT", "")
RUNNER = os.path.join(OUT, "libref_runner.so")

# (N, dt, gravity multiplier) of the cases the tests and bench use
CONFIGS = [
    (64, 0.01, 1.0),
    (128, 0.005, 1.0),
    (512, 0.002, 1.0),
    (2048, 0.001, 1.0),
    (4096, 0.001, 1.0),
    (8192, 0.0005, 1.0),
]


def ptx_path(N: int, dt: float, g: float = 1.0) -> str:
    return os.path.join(OUT, f"ref_N{N}_dt{dt!r}_g{g!r}.ptx")


def _nvcc() -> str | None:
    return shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)


def reference_present() -> bool:
    return bool(REFERENCE_ROOT) and os.path.exists(os.path.join(REFERENCE_ROOT, "CosmosCuda.cuh"))


def build_ptx(force: bool = False) -> list[str]:
    nvcc = _nvcc()
    if not nvcc or not reference_present():
        return []
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(HERE, "ref_kernels.cu")
    jobs = []
    for N, dt, g in CONFIGS:
        out = ptx_path(N, dt, g)
        if not force and os.path.exists(out) and os.path.getmtime(out) > os.path.getmtime(src):
            continue
        jobs.append([nvcc, "-ptx", "-arch=compute_103a", "-O3", "--use_fast_math", "-std=c++17",
                     f"-DREF_N={N}", f"-DREF_DT={dt!r}f", f"-DREF_G={g!r}f", "-I", REFERENCE_ROOT, src, "-o", out])

    def run(cmd):
        return subprocess.run(cmd, capture_output=True, text=True)

    with cf.ThreadPoolExecutor(max_workers=4) as ex:
        for cmd, r in zip(jobs, ex.map(run, jobs)):
            if r.returncode != 0:
                sys.stderr.write(r.stdout + r.stderr)
                raise RuntimeError("reference PTX build failed: " + " ".join(cmd))
    return [ptx_path(*c) for c in CONFIGS]


def build_runner(force: bool = False) -> str | None:
    nvcc = _nvcc()
    if not nvcc:
        return None
    src = os.path.join(HERE, "ref_runner.cpp")
    if not force and os.path.exists(RUNNER) and os.path.getmtime(RUNNER) > os.path.getmtime(src):
        return RUNNER
    os.makedirs(OUT, exist_ok=True)
    cuda = os.path.dirname(os.path.dirname(nvcc))
    cmd = [nvcc, "-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", src, "-o", RUNNER,
           "-L", os.path.join(cuda, "lib64"), "-L", os.path.join(cuda, "lib64", "stubs"),
           "-lcuda", "-lcufft", "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("reference runner build failed")
    return RUNNER


def build_if_available() -> None:
    build_ptx()
    build_runner()


if __name__ == "__main__":
    print(build_ptx(force="--force" in sys.argv), build_runner(force="--force" in sys.argv))
