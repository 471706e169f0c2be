"""Build libamps.so (CUDA kernels + C ABI) in-tree for sm_103a.

    python -m w3914777_gb300.build        # or: from w3914777_gb300.build import build; build()

Each translation unit is compiled by its own nvcc process (in parallel), then
linked into w3914777_gb300/_lib/libamps.so with the CUDA runtime linked
statically, so the library needs nothing but the driver at run time.
"""
import os
import platform
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libamps.so")
OBJ = os.path.join(OUT, "obj-" + platform.machine())
_ELF_MACHINE = {"x86_64": 62, "aarch64": 183}

SOURCES = ["amps_api.cu", "amps_host.cpp", "k_common.cu", "k_graingrowth.cu", "k_gg_half.cu", "k_gg_ragged.cu",
           "k_gg_ensemble.cu", "k_kobayashi.cu",
           "k_sintering.cu", "k_sint_ref.cu", "k_noalloc.cu", "k_adjoint.cu", "k_diag.cu", "compat.cu",
           "compat_half.cu"]
# per-file flags: the reference-named kernels keep the reference's rounding (no fused multiply-add)
FILE_FLAGS = {"compat.cu": ["-fmad=false"]}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include")]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def foreign_binary(path):
    """True if `path` is an ELF file built for another machine than this one."""
    want = _ELF_MACHINE.get(platform.machine())
    try:
        with open(path, "rb") as f:
            head = f.read(20)
    except OSError:
        return False
    if want is None or len(head) < 20 or head[:4] != b"\x7fELF":
        return False
    return int.from_bytes(head[18:20], "little") != want


def build(verbose=False, force=False, extra_flags=()):
    os.makedirs(OBJ, exist_ok=True)
    for path in (LIB, os.path.join(ROOT, "oracle", "liboracle.so"), os.path.join(ROOT, "oracle", "liboracle_fast.so")):
        if foreign_binary(path):
            os.remove(path)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers += [os.path.join(ROOT, "include", h) for h in ("amps.h", "amps_compat.h")]
    cc = nvcc()
    jobs = []
    objs = []
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(OBJ, src + ".o")
        objs.append(obj)
        if force or _newer(obj, [path] + headers):
            cmd = [cc, *ARCH, *NVCC_FLAGS, *FILE_FLAGS.get(src, []), *extra_flags, "-c", path, "-o", obj]
            if src.endswith(".cpp"):
                cmd = [cc, *NVCC_FLAGS, "-x", "c++", "-c", path, "-o", obj]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.returncode

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        rcs = list(ex.map(run, jobs))
    if any(rcs):
        raise RuntimeError("nvcc failed")
    if jobs or not os.path.exists(LIB):
        cmd = [cc, *ARCH, "-shared", "-o", LIB, *objs, "-cudart", "static", "-Xcompiler", "-fPIC"]
        if run(cmd):
            raise RuntimeError("link failed")
    build_drivers(cc, run, force or bool(jobs))
    return LIB


DRIVER_SRC = os.path.join(HERE, "drivers", "amps_driver.cpp")
DRIVER = os.path.join(OUT, "amps_driver")
DRIVER_NAMES = ["snowflake_purehigh", "snowflake_purelow", "snowflake_end2end_mix", "graingrowth_purehigh",
                "graingrowth_purelow", "graingrowth_end2end_mix", "sintering_main"]


def build_drivers(cc, run, force=False):
    """The reference's driver programs (one executable, one name per program)."""
    if foreign_binary(DRIVER):
        os.remove(DRIVER)
    if force or _newer(DRIVER, [DRIVER_SRC, LIB, os.path.join(ROOT, "include", "amps.h")]):
        cmd = [cc, "-O2", "-std=c++17", "-x", "cu", DRIVER_SRC, "-o", DRIVER, "-L" + OUT, "-lamps",
               "-Xlinker", "-rpath,$ORIGIN", "-cudart", "static"]
        if run(cmd):
            raise RuntimeError("driver build failed")
    for name in DRIVER_NAMES:
        link = os.path.join(OUT, name)
        if not os.path.islink(link):
            if os.path.exists(link):
                os.remove(link)
            os.symlink("amps_driver", link)


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
