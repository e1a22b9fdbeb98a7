"""In-tree build of the native libraries (no pip install, no cmake).

libsps_gb300.so  -- CUDA kernels for sm_103a + the C-ABI of include/sps.h
libsph_host.so   -- host-side set-up library of include/sph_host.h
sps_run          -- the reference's main program over the C-ABI (a driver executable)

The FP64 plain kernels are compiled with -fmad=false and all host code with
-ffp-contract=off: the reference (gfortran -O3 on x86-64) never fuses a multiply with an
add, and the plain mode reproduces its rounding on either host architecture.
"""
import os
import subprocess
import concurrent.futures as cf

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(PKG_DIR))
CSRC = os.path.join(os.path.dirname(PKG_DIR), "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIB_DIR = os.path.join(PKG_DIR, "lib")
OBJ_DIR = os.path.join(LIB_DIR, "obj")

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# (source, extra nvcc flags)
CUDA_UNITS = [
    ("cuda/sps_api.cu", []),
    ("cuda/neighbours.cu", ["-fmad=false"]),
    ("cuda/plain_step.cu", ["-fmad=false"]),
    ("cuda/fast_step.cu", []),
    ("cuda/surface.cu", ["-fmad=false"]),
    ("cuda/mlp_train.cu", []),
    ("cuda/mlp_tc.cu", []),
    ("cuda/neighbour_stats_static.cu", ["-fmad=false"]),
]


def lib_path(name):
    return os.path.join(LIB_DIR, name)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def _headers():
    hs = [os.path.join(INCLUDE, h) for h in os.listdir(INCLUDE)]
    cdir = os.path.join(CSRC, "cuda")
    hs += [os.path.join(cdir, h) for h in os.listdir(cdir) if h.endswith((".cuh", ".h"))]
    return hs


def build_host(force=False):
    os.makedirs(LIB_DIR, exist_ok=True)
    src = os.path.join(CSRC, "host", "sph_problem.cpp")
    out = lib_path("libsph_host.so")
    if not force and _newer(out, [src] + _headers()):
        return out
    # -ffp-contract=off: the set-up arithmetic must not fuse multiply-adds (aarch64 GCC
    # contracts by default; the reference's x86-64 build has no FMA)
    _run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-Wall",
          "-I" + INCLUDE, "-o", out, src])
    return out


def build_cuda(force=False, verbose=False):
    os.makedirs(OBJ_DIR, exist_ok=True)
    out = lib_path("libsps_gb300.so")
    srcs = [os.path.join(CSRC, s) for s, _ in CUDA_UNITS]
    if not force and _newer(out, srcs + _headers()):
        return out
    jobs = []
    for s, extra in CUDA_UNITS:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJ_DIR, os.path.basename(s) + ".o")
        cmd = [NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                               "-Xcompiler", "-ffp-contract=off",
                               "-Xptxas", "-v" if verbose else "-O3", "-I" + INCLUDE,
                               "-I" + os.path.join(CSRC, "cuda"), "-c", src, "-o", obj] + extra
        jobs.append((cmd, obj))
    logs = []
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        for log in ex.map(lambda j: _run(j[0]), jobs):
            logs.append(log)
    _run([NVCC] + ARCH + ["-shared", "-o", out] + [o for _, o in jobs] + ["-lcudart"])
    if verbose:
        print("\n".join(logs))
    return out


def build_driver(force=False):
    """sps_run: the reference's main program over the C-ABI (csrc/host/sps_run.cpp), linked
    against the two libraries beside it."""
    src = os.path.join(CSRC, "host", "sps_run.cpp")
    out = lib_path("sps_run")
    libs = [lib_path("libsps_gb300.so"), lib_path("libsph_host.so")]
    if not force and _newer(out, [src] + libs + _headers()):
        return out
    # the linker resolves libsps_gb300.so's own dependency (the CUDA runtime) in the
    # toolkit's library directory
    cuda_lib = os.path.join(os.path.dirname(os.path.dirname(NVCC)), "lib64")
    _run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-Wall", "-I" + INCLUDE, "-o", out,
          src, "-L" + LIB_DIR, "-lsps_gb300", "-lsph_host", "-Wl,-rpath,$ORIGIN",
          "-Wl,-rpath-link," + cuda_lib])
    return out


def build_all(force=False, verbose=False):
    """The two libraries, then the driver.  The libraries are the product: a driver that
    fails to link is reported on stderr and does not stop their build (build_driver itself
    raises, and its test calls it directly)."""
    host, cuda = build_host(force), build_cuda(force, verbose)
    try:
        driver = build_driver(force)
    except RuntimeError as e:
        import sys
        print("sps_gb300: the sps_run driver was not built: %s" % e, file=sys.stderr)
        driver = None
    return host, cuda, driver
