"""Builds libmatfun_cuda.so (sm_103a) in-tree from matfun_gb300/csrc, and the CPU oracle library used by the tests.

    python -m matfun_gb300.build            (or __graft_entry__.build())

The kernel translation units (one per family and kind) are compiled in parallel with nvcc and linked into
matfun_gb300/libmatfun_cuda.so.  Objects go to matfun_gb300/_build/ and are reused while no source changed.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmatfun_cuda.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-warn-spills"]


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmatfun_cuda")


def _elf_native(path):
    """True if path is an ELF file for this machine (objects built on another host architecture are rebuilt)"""
    import platform
    want = {"x86_64": 62, "aarch64": 183, "arm64": 183}.get(platform.machine())
    try:
        with open(path, "rb") as f:
            h = f.read(20)
    except OSError:
        return False
    if len(h) < 20 or h[:4] != b"\x7fELF":
        return False
    return want is None or int.from_bytes(h[18:20], "little") == want


def _fresh(out, inputs_time):
    return os.path.exists(out) and _elf_native(out) and os.path.getmtime(out) >= inputs_time


def _newest_header():
    hs = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
    hs += glob.glob(os.path.join(ROOT, "include", "*.h"))
    return max((os.path.getmtime(h) for h in hs), default=0.0)


def _rdc(src):
    """the batched kernel and its tile routines: relocatable device code, device-linked together"""
    return os.path.basename(src).startswith("batched")


def _extra(src):
    """the general family's batched tile routines: 168 registers (65536 / (128 threads x 3 CTAs per SM)), so that
    batched_gmf_kernel runs 3 CTAs per SM like the standalone gmf kernel, whose launch bounds give the same"""
    return ["-maxrregcount=168"] if os.path.basename(src) in ("batched_gmf.cu", "batched_gmf32.cu") else []


def _compile(src, hdr_time, verbose):
    obj = os.path.join(OBJ, os.path.basename(src)[:-3] + ".o")
    if _fresh(obj, max(os.path.getmtime(src), hdr_time)):
        return obj, ""
    cmd = [_nvcc()] + NVFLAGS + (["-rdc=true"] if _rdc(src) else []) + _extra(src) + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, (r.stdout + r.stderr) if verbose else ""


def build_cuda(verbose=False, jobs=None):
    os.makedirs(OBJ, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdr = max(_newest_header(), os.path.getmtime(__file__))  # (the compiler flags live in this file)
    jobs = jobs or max(1, min(len(srcs), os.cpu_count() or 4))
    with cf.ThreadPoolExecutor(jobs) as ex:
        res = list(ex.map(lambda s: _compile(s, hdr, verbose), srcs))
    objs = [o for o, _ in res]
    for _, log in res:
        if log:
            print(log)
    rdc = [o for s, o in zip(srcs, objs) if _rdc(s)]
    if rdc:
        dl = os.path.join(OBJ, "device_link.o")
        if not _fresh(dl, max(os.path.getmtime(o) for o in rdc)):
            r = subprocess.run([_nvcc()] + ARCH + ["-Xcompiler", "-fPIC", "-dlink", "-o", dl] + rdc,
                               capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"device link failed:\n{r.stdout}\n{r.stderr}")
        objs = objs + [dl]
    if not _fresh(LIB, max(os.path.getmtime(o) for o in objs)):
        tmp = LIB + ".tmp"
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


def build_shim():
    """matfun_gb300/libmatfun.so: the reference's CPU API names (include/matfun.h) forwarding to libmatfun_cuda.so"""
    src = os.path.join(HERE, "shim", "matfun_shim.c")
    lib = os.path.join(HERE, "libmatfun.so")
    if _fresh(lib, max(os.path.getmtime(src), os.path.getmtime(LIB))):
        return lib
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-o", lib + ".tmp", src, "-L" + HERE, "-l:libmatfun_cuda.so",
           "-Wl,-rpath,$ORIGIN"]
    subprocess.run(cmd, check=True)
    os.replace(lib + ".tmp", lib)
    return lib


def build_oracle():
    """the CPU restatement (oracle/oracle.c) as oracle/liboracle.so: test infrastructure, never the product path"""
    src = os.path.join(ROOT, "oracle", "oracle.c")
    lib = os.path.join(ROOT, "oracle", "liboracle.so")
    if _fresh(lib, os.path.getmtime(src)):
        return lib
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-fno-math-errno", "-fno-trapping-math",
           "-o", lib + ".tmp", src, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(lib + ".tmp", lib)
    return lib


REF_OUT = os.path.join(ROOT, "oracle", "_ref")
REF_ROOT_FILE = os.path.join(REF_OUT, "REFERENCE_ROOT")  # the tree the last build_reference_oracle used


def _is_reference_tree(path):
    return bool(path) and os.path.isdir(os.path.join(path, "c", "src"))


def reference_root():
    """the reference source tree, where it is present: the MATFUN_REFERENCE_ROOT environment variable, else the tree
    the reference oracle was last built from (recorded by build_reference_oracle); None on hosts without it"""
    cand = [os.environ.get("MATFUN_REFERENCE_ROOT")]
    try:
        with open(REF_ROOT_FILE) as f:
            cand.append(f.read().strip())
    except OSError:
        pass
    return next((c for c in cand if _is_reference_tree(c)), None)


def build_reference_oracle(ref):
    """the reference's own CPU library (oracle/_ref/libmatfun_ref.so) and its CUDA kernels as an sm_103a cubin
    (oracle/_ref/matfun_cuda_ref.cubin), built from the reference tree `ref` where it lies; the library's sources are
    also staged into oracle/_ref/src (never committed) so that a host without the tree builds the same library from
    them.  On such a host (`ref` is not a reference tree) the library is built from the staged sources, the cubin
    having travelled with the working tree.  None when neither is present."""
    staged = os.path.join(REF_OUT, "src")
    mk = ["make", "-s", "-f", os.path.join("oracle", "Makefile.ref")]
    if _is_reference_tree(ref):
        subprocess.run(mk + [f"REF={ref}", "all", "stage"], cwd=ROOT, check=True)
        with open(REF_ROOT_FILE, "w") as f:
            f.write(os.path.abspath(ref) + "\n")
    elif _is_reference_tree(staged):
        subprocess.run(mk + [f"REF={staged}", "lib"], cwd=ROOT, check=True)
    else:
        return None
    return os.path.join(REF_OUT, "libmatfun_ref.so")


def build_ref_gpu_timer():
    """oracle/ref_gpu_timer.so: launcher of the reference's cubin (test and benchmark infrastructure)"""
    src = os.path.join(ROOT, "oracle", "ref_gpu_timer.cu")
    lib = os.path.join(ROOT, "oracle", "ref_gpu_timer.so")
    if _fresh(lib, os.path.getmtime(src)):
        return lib
    cmd = [_nvcc(), "-shared", "-Xcompiler", "-fPIC", "-O2", "-o", lib + ".tmp", src, "-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"ref_gpu_timer build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(lib + ".tmp", lib)
    return lib


if __name__ == "__main__":
    print(build_cuda(verbose=True))
    print(build_shim())
    print(build_oracle())
