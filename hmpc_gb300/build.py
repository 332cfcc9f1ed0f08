"""Build libhmpc_gb300.so in-tree for sm_103a.

One translation unit per limb count (kernels.cu with -DHMPC_L=1..9) plus the
host-side C-ABI layer; the units compile in parallel and only the ones whose
sources changed are rebuilt.  The benchmark's rate probes (probe.cu) link into
a library of their own, libhmpc_gb300_probes.so, outside the product's ABI.
"""
import concurrent.futures
import os
import pathlib
import shutil
import subprocess

HERE = pathlib.Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT = HERE / "_build"
LIB = OUT / "libhmpc_gb300.so"
PROBES = OUT / "libhmpc_gb300_probes.so"
INCLUDE = HERE.parent / "include"
LIMBS = range(1, 10)
TC_LIMBS = range(2, 9)  # limb counts of the tensor-core transform
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build hmpc_gb300")
    return path


def _headers():
    return list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.hpp")) + [INCLUDE / "hmpc_gb300.h"]


def _stale(target, sources):
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def _run(cmd):
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(map(str, cmd))}\n{proc.stdout}\n{proc.stderr}")
    return proc.stderr


def build(verbose=False, jobs=None):
    OUT.mkdir(exist_ok=True)
    headers = _headers()
    common = [nvcc(), "-std=c++17", "-O3", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC", "-I", str(INCLUDE)]
    steps = []
    objects = []
    for limbs in LIMBS:
        obj = OUT / f"kernels_L{limbs}.o"
        objects.append(obj)
        if _stale(obj, [CSRC / "kernels.cu", *headers]):
            steps.append(common + [f"-DHMPC_L={limbs}", "-c", str(CSRC / "kernels.cu"), "-o", str(obj)])
    for limbs in TC_LIMBS:
        obj = OUT / f"tensor_ntt_L{limbs}.o"
        objects.append(obj)
        if _stale(obj, [CSRC / "tensor_ntt.cu", *headers]):
            steps.append(common + [f"-DHMPC_L={limbs}", "-c", str(CSRC / "tensor_ntt.cu"), "-o", str(obj)])
    probe_obj = OUT / "probe.o"
    if _stale(probe_obj, [CSRC / "probe.cu", *headers]):
        steps.append(common + ["-c", str(CSRC / "probe.cu"), "-o", str(probe_obj)])
    for name in ("api.cpp", "host_math.cpp", "noalloc.cu", "batched.cpp", "serve.cpp", "cipher.cu",
                 "tc.cpp", "wire.cu", "linalg.cpp"):
        obj = OUT / (name.rsplit(".", 1)[0] + ".o")
        objects.append(obj)
        if _stale(obj, [CSRC / name, *headers]):
            steps.append(common + ["-x", "cu", "-c", str(CSRC / name), "-o", str(obj)])
    jobs = jobs or min(len(steps) or 1, os.cpu_count() or 4)
    with concurrent.futures.ThreadPoolExecutor(max_workers=jobs) as pool:
        for log in pool.map(_run, steps):
            if verbose and log:
                print(log)
    if steps or _stale(LIB, objects):
        _run([nvcc(), "-shared", *ARCH, "-o", str(LIB), *map(str, objects), "-lcudart"])
    if _stale(PROBES, [probe_obj]):
        _run([nvcc(), "-shared", *ARCH, "-o", str(PROBES), str(probe_obj), "-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
