"""Build libjx.so (the sm_103a kernels and their C ABI) in place with nvcc.

Each ``csrc/*.cu`` is compiled to an object in parallel, then linked into
``jathenax_gb300/libjx.so``. Run as ``python -m jathenax_gb300.build``; the
repository's ``__graft_entry__.build()`` calls :func:`build`.
"""

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PACKAGE = Path(__file__).resolve().parent
CSRC = PACKAGE / "csrc"
LIBRARY = PACKAGE / "libjx.so"
OBJDIR = PACKAGE / "_build"
ARCH = ("-gencode", "arch=compute_103a,code=sm_103a")


def nvcc_path():
    for candidate in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if candidate and Path(candidate).exists():
            return candidate
    raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libjx.so")


def _compile(nvcc, source, flags):
    obj = OBJDIR / (source.stem + ".o")
    cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-I", str(PACKAGE.parent / "include"), *flags, "-c", str(source), "-o", str(obj)]
    result = subprocess.run(cmd, capture_output=True, text=True)
    if result.returncode != 0:
        raise RuntimeError(f"nvcc failed on {source.name}:\n{result.stdout}\n{result.stderr}")
    return obj, result.stderr


def _compile_host(source):
    """Host C++ (no device code), without FMA contraction so results match Python."""
    obj = OBJDIR / (source.stem + ".o")
    cxx = os.environ.get("CXX") or shutil.which("g++") or "c++"
    cmd = [cxx, "-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-c", str(source), "-o", str(obj)]
    result = subprocess.run(cmd, capture_output=True, text=True)
    if result.returncode != 0:
        raise RuntimeError(f"{cxx} failed on {source.name}:\n{result.stdout}\n{result.stderr}")
    return obj, result.stderr


def build(verbose=False, ptxas_info=False, jobs=None):
    """Compile every kernel for sm_103a and link libjx.so; returns its path."""
    nvcc = nvcc_path()
    OBJDIR.mkdir(exist_ok=True)
    # The longest translation units (the WENO-Z and PPMX kernels) go first,
    # so that the pool does not end on one of them.
    sources = sorted(CSRC.glob("*.cu"), key=lambda f: (0 if "wenoz" in f.stem else 1 if "ppmx" in f.stem else 2, f.name))
    host_sources = sorted(CSRC.glob("*.cpp"))
    flags = ["-Xptxas", "-v"] if ptxas_info else []
    jobs = jobs or min(len(sources) + len(host_sources), os.cpu_count() or 4)
    with ThreadPoolExecutor(max_workers=jobs) as pool:
        futures = [pool.submit(_compile, nvcc, s, flags) for s in sources]
        futures += [pool.submit(_compile_host, s) for s in host_sources]
        results = [f.result() for f in futures]
    objects = [obj for obj, _ in results]
    if verbose or ptxas_info:
        for _, log in results:
            if log:
                sys.stderr.write(log)
    tmp = LIBRARY.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objects), "-lcudart"]
    result = subprocess.run(cmd, capture_output=True, text=True)
    if result.returncode != 0:
        raise RuntimeError(f"link failed:\n{result.stdout}\n{result.stderr}")
    os.replace(tmp, LIBRARY)
    return LIBRARY


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="-v" in sys.argv))
