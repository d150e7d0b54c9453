"""Build ``libgbspec.so`` in tree with nvcc (sm_103a only).

``python -m fluidsim_gb300.build`` compiles each ``csrc/*.cu`` translation
unit in parallel and links the shared library next to this file.  Objects
go to ``fluidsim_gb300/_build``; both are git-ignored build products.
"""

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIB = HERE / "libgbspec.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["gbs_fft.cu", "gbs_ns.cu", "gbs_noalloc.cu", "gbs_fast_f32.cu", "gbs_fast_f64.cu",
           "gbs_turb.cu", "gbs_mlp.cu", "gbs_les.cu",
           "gbs_ensemble.cu", "gbs_spectra.cu", "gbs_forcing.cu"]


def nvcc_path():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required")
    return cand


def _needs_rebuild(obj, src):
    if not obj.exists():
        return True
    stamp = obj.with_suffix(".flags")
    if not stamp.exists() or stamp.read_text() != os.environ.get("GBS_NVCC_FLAGS", ""):
        return True
    deps = ([src] + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h"))
            + [HERE.parent / "include" / "gbspec.h"])
    return any(d.stat().st_mtime > obj.stat().st_mtime for d in deps)


def build(verbose=False, force=False):
    nvcc = nvcc_path()
    BUILD.mkdir(exist_ok=True)
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                    "-I", str(HERE.parent / "include")]
    extra = os.environ.get("GBS_NVCC_FLAGS", "").split()
    flags += extra

    def compile_one(name):
        src = CSRC / name
        obj = BUILD / (name + ".o")
        if not force and not _needs_rebuild(obj, src):
            return obj
        cmd = [nvcc] + flags + ["-c", str(src), "-o", str(obj)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}:\n{res.stderr}")
        if verbose:
            print(res.stderr, file=sys.stderr)
        obj.with_suffix(".flags").write_text(os.environ.get("GBS_NVCC_FLAGS", ""))
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    if force or not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc] + ARCH + ["-shared", "-o", str(tmp)] + [str(o) for o in objs] + [
            "-cudart", "static"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
