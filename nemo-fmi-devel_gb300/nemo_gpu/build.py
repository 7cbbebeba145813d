"""Build recipe of the CUDA library (sm_103a only).

Seven translation units are compiled in parallel and linked into
``nemo_gpu/_lib/libnemo_gpu.so``:

* ``inst_fp64.cu`` -- FP64 kernels, ``--fmad=false`` so that every double operation
  rounds exactly like the reference's FP64 CPU build (no fused multiply-add);
* ``inst_fp32.cu`` -- FP32-bulk kernels of the mixed-precision mode, with
  ``--prec-div=false`` (single-precision quotients within 2 ulp instead of
  correctly rounded: the mixed form's tolerance is set by FP32 storage, and the
  correctly rounded quotient costs a multi-instruction sequence per division);
* ``capi.cu``      -- the C ABI (host code; the host compiler without contraction,
  ``-ffp-contract=off``, so that the scalars it forms -- barotropic weights, the
  EOS-80 re-expansion, the forcing's seasonal factors -- round like the oracle's on
  any host, FMA-capable Arm included);
* ``noalloc.cu``   -- the allocation-free global sum (static device scratch);
* ``adj_fp64.cu``  -- the adjoint kernels of the tracer routines and tra_nxt
  (``--fmad=false``);
* ``inst_step.cu`` -- the rest of the model step (wzv, dyn_zdf, dyn_nxt, ssh_swp,
  the momentum trends, eos, zdf_phy, the forcing, stp_ctl, dia_hsb, the z* time
  stepping, ...), both precisions (``--fmad=false``);
* ``inst_triad.cu`` -- the triad operator (ldf_slp_triad, tra_ldf_triad), both
  precisions (``--fmad=false``).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)
CSRC = os.path.join(ROOT, "csrc")
OBJ_DIR = os.path.join(ROOT, "_build")
LIB_DIR = os.path.join(PKG_DIR, "_lib")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "--extended-lambda", "-lineinfo", "-Xcompiler", "-fPIC"]
UNITS = {
    "inst_fp64.cu": ["--fmad=false"],
    "inst_fp32.cu": ["--prec-div=false"],
    "capi.cu": ["-Xcompiler", "-ffp-contract=off"],
    "noalloc.cu": ["--fmad=false"],
    "adj_fp64.cu": ["--fmad=false"],
    "inst_step.cu": ["--fmad=false"],
    "inst_triad.cu": ["--fmad=false"],
}


def library_path():
    return os.path.join(LIB_DIR, "libnemo_gpu.so")


def _nvcc():
    nv = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nv):
        raise RuntimeError("nvcc not found")
    return nv


def _sources_newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    """Compile the CUDA library if any source is newer than it; return its path."""
    os.makedirs(OBJ_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(os.path.dirname(ROOT), "include", "nemo_gpu.h"))
    nvcc = _nvcc()
    jobs = []
    for unit, extra in UNITS.items():
        src = os.path.join(CSRC, unit)
        obj = os.path.join(OBJ_DIR, unit.replace(".cu", ".o"))
        if force or _sources_newer(obj, [src] + headers):
            jobs.append([nvcc] + ARCH + COMMON + extra + ["-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose:
            print(" ".join(cmd))
        return r

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(OBJ_DIR, u.replace(".cu", ".o")) for u in UNITS]
    lib = library_path()
    if force or jobs or _sources_newer(lib, objs):
        run([nvcc] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart"])
    return lib
