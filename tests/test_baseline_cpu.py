"""The host driver of the reference's own CUDA kernels (baseline/ref_cuda.cpp)
builds and exports its entry points (no GPU call here); the cubins it loads
need the reference tree and are checked on the GPU
(tests/test_gpu_reference_cuda.py)."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "baseline", "_ref", "libref_cuda.so")


def test_host_driver_builds_and_exports_its_entry_points():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "baseline"), "loader"], check=True)
    # the symbol table (loading it needs the CUDA driver library, absent on a machine without a GPU)
    out = subprocess.run(["nm", "-D", "--defined-only", LIB], check=True, capture_output=True, text=True).stdout
    names = {line.split()[-1] for line in out.splitlines() if line.strip()}
    for name in ("refcuda_error", "refcuda_open", "refcuda_close", "refcuda_dims", "refcuda_gg_pure",
                 "refcuda_gg_mix", "refcuda_kob_pure", "refcuda_kob_mix", "refcuda_sint_pure", "refcuda_sint_mix",
                 "refcuda_gg_purelow", "refcuda_kob_purelow"):
        assert name in names, name
