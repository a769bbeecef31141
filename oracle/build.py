"""Build recipe for the oracle — TEST INFRASTRUCTURE ONLY.

build_oracle():    oracle/pointcloud.c -> oracle/_build/liboracle.so (gcc, -O2,
                   -ffp-contract=off so float results match the reference's
                   operation order exactly).
build_reference(): when the reference tree is present, compiles the
                   reference's own point-cloud library source where it lies
                   (OpenHolo_KETI/.../ophgen_pointcloud/ophgen_pointcloud.cpp)
                   together with oracle/keti_ref_harness.cpp into
                   oracle/_ref/libketi_ref.so (sequential; the reference's
                   OpenMP loop races on its output) and
                   oracle/_ref/libketi_ref_omp.so (-fopenmp, timing only).
                   Nothing is copied out of the reference tree.
build_reference_depthmap():
                   when the reference tree is present, compiles the device
                   code of the reference's depth-map kernels
                   (OpenHolo_DepthMap/Hologram/src/HologramKernel.cu), where
                   it lies, into oracle/_ref/dm_ref.cubin for sm_103a, and
                   records the entry names ptxas reports in
                   oracle/_ref/dm_ref_entries.txt.  oracle/dm_reference.py runs
                   these kernels on a GPU in the reference's call sequence.
                   The depth-map host code (Qt, FFTW) and the WRP sources (the
                   closed CWO DLL) are not built.
build_reference_pointcloud_gpu():
                   when the reference tree is present, compiles the device
                   code of the reference's point-cloud GPU library
                   (OpenHolo_KETI/.../ophgen_pointcloud_gpu/ophgen_pointcloud_gpu.cpp,
                   CUDA source in a .cpp file, so nvcc -x cu), where it lies,
                   into oracle/_ref/pc_ref.cubin for sm_103a.
                   oracle/pc_reference_gpu.py launches its kernel as the
                   reference's host function does.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
REFERENCE_ROOT = Path(os.environ.get("OH_REFERENCE_ROOT", "/root/reference"))
KETI_DIR = REFERENCE_ROOT / "OpenHolo_KETI/VS/Openholo_Generation_PointCloud_Library_beta_v1.0/ophgen_pointcloud"


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")


def _fresh(out: Path, deps) -> bool:
    return out.exists() and all(out.stat().st_mtime >= Path(d).stat().st_mtime for d in deps)


def build_oracle() -> Path:
    BUILD.mkdir(exist_ok=True)
    out = BUILD / "liboracle.so"
    src = HERE / "pointcloud.c"
    if not _fresh(out, [src]):
        _run(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-o", str(out), str(src), "-lm"])
    return out


def build_reference() -> Path | None:
    src = KETI_DIR / "ophgen_pointcloud.cpp"
    if not src.exists():
        return None
    REF_OUT.mkdir(exist_ok=True)
    harness = HERE / "keti_ref_harness.cpp"
    outs = {"libketi_ref.so": [], "libketi_ref_omp.so": ["-fopenmp"]}
    for name, extra in outs.items():
        out = REF_OUT / name
        if _fresh(out, [src, harness]):
            continue
        _run(["g++", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-w", *extra, "-I", str(KETI_DIR),
              "-o", str(out), str(src), str(harness)])
    return REF_OUT / "libketi_ref.so"


DM_KERNEL_SRC = REFERENCE_ROOT / "OpenHolo_DepthMap/Hologram/src/HologramKernel.cu"


def build_reference_depthmap() -> Path | None:
    src = DM_KERNEL_SRC
    if not src.exists():
        return None
    REF_OUT.mkdir(exist_ok=True)
    out = REF_OUT / "dm_ref.cubin"
    names = REF_OUT / "dm_ref_entries.txt"
    if _fresh(out, [src]) and names.exists():
        return out
    nvcc = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
    r = subprocess.run([nvcc, "-cubin", "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "-Xptxas", "-v", "-w",
                        "-o", str(out), str(src)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    entries = []
    for line in (r.stdout + r.stderr).splitlines():
        if "Compiling entry function '" in line:
            entries.append(line.split("'")[1])
    names.write_text("\n".join(sorted(set(entries))) + "\n")
    return out


KETI_GPU_SRC = REFERENCE_ROOT / ("OpenHolo_KETI/VS/Openholo_Generation_PointCloud_Library_beta_v1.0/"
                                 "ophgen_pointcloud_gpu/ophgen_pointcloud_gpu.cpp")


def build_reference_pointcloud_gpu() -> Path | None:
    src = KETI_GPU_SRC
    if not src.exists():
        return None
    REF_OUT.mkdir(exist_ok=True)
    out = REF_OUT / "pc_ref.cubin"
    if _fresh(out, [src]):
        return out
    nvcc = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
    _run([nvcc, "-x", "cu", "-cubin", "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "-w",
          "-I", str(src.parent), "-I", str(KETI_DIR), "-o", str(out), str(src)])
    return out


if __name__ == "__main__":
    print(build_oracle())
    print(build_reference())
    print(build_reference_depthmap())
    print(build_reference_pointcloud_gpu())
