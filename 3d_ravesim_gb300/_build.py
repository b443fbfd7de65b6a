"""Build librs_fresnel.so from csrc/*.cu with nvcc for sm_103a (in-tree, no cmake).

Each translation unit is compiled in parallel, then linked into a shared library with the
C ABI declared in include/rs_fresnel.h. The library is rebuilt when any source or header is
newer than it.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
# RS_BUILD_DIR / RS_NVCC_EXTRA select another output directory and extra nvcc flags (e.g. a
# -DRS_PACKED_F32X2=0 variant built side by side for comparison).
BUILD = Path(os.environ.get("RS_BUILD_DIR", PKG / "_build"))
LIB = BUILD / "librs_fresnel.so"
SOURCES = ["rs_pass_pow2_rows.cu", "rs_pass_pow2_cols.cu", "rs_pass_pow3_rows.cu", "rs_pass_pow3_cols.cu", "rs_pass_x2.cu",
           "rs_dispatch.cu", "rs_misc.cu", "rs_abi.cu"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    return "nvcc"


def common_flags() -> list[str]:
    return [
        "-std=c++17", "-O3", ARCH, "-lineinfo",
        "-Xcompiler", "-fPIC,-ffp-contract=off",
        f"-I{INCLUDE}", f"-I{CSRC}",
        *os.environ.get("RS_NVCC_EXTRA", "").split(),
    ]


def _stale() -> bool:
    if not LIB.exists():
        return True
    flags_file = BUILD / "flags.txt"
    if not flags_file.exists() or flags_file.read_text() != " ".join(common_flags()):
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile (if needed) and return the path of librs_fresnel.so."""
    if not force and not _stale():
        return LIB
    BUILD.mkdir(exist_ok=True)
    cc = nvcc()

    def compile_one(src: str) -> tuple[str, int, str]:
        obj = BUILD / (Path(src).stem + ".o")
        cmd = [cc, *common_flags(), "-c", str(CSRC / src), "-o", str(obj)]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        return src, r.returncode, r.stdout + r.stderr

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(compile_one, SOURCES))
    for src, rc, out in results:
        if rc != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{out}")
        if verbose and out:
            sys.stderr.write(out)
    tmp = BUILD / "librs_fresnel.so.tmp"
    link = [cc, "-shared", ARCH, "-cudart", "shared", "-Xlinker", "-rpath,/usr/local/cuda/lib64",
            "-o", str(tmp), *[str(BUILD / (Path(s).stem + ".o")) for s in SOURCES]]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}{r.stderr}")
    os.replace(tmp, LIB)
    (BUILD / "flags.txt").write_text(" ".join(common_flags()))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
