"""Builds liblivre_gb300.so: the sm_103a CUDA kernels and the C-ABI host runtime.

Each .cu translation unit is compiled by nvcc in parallel (one -gencode,
sm_103a) and linked with the static CUDA runtime into
livre_gb300/_build/liblivre_gb300.so. Host code is compiled with
-ffp-contract=off so the host-side frustum math is plain IEEE single
precision on x86_64 and aarch64 alike.
"""
import concurrent.futures as cf
import hashlib
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liblivre_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".h")]
    hs.append(os.path.join(ROOT, "include", "livre_gb300.h"))
    return hs


def _flags():
    return ["-O3", "-std=c++17", "-lineinfo", *ARCH, "-I", os.path.join(ROOT, "include"),
            "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math", "--expt-relaxed-constexpr"]


def _digest():
    h = hashlib.sha1()
    for p in sources() + headers() + [__file__]:
        h.update(open(p, "rb").read())
    h.update(" ".join(_flags()).encode())
    return h.hexdigest()


def _compile(src):
    obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
    cmd = [NVCC, *_flags(), "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    return obj


def build(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    stamp = os.path.join(OUT_DIR, "stamp")
    dig = _digest()
    if not force and os.path.exists(LIB) and os.path.exists(stamp) and open(stamp).read() == dig:
        return LIB
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, sources()))
    tmp = LIB + ".tmp%d" % os.getpid()
    # the soname lets a plugin library linked with -llivre_gb300 bind to the
    # copy already loaded (one source registry per process)
    cmd = [NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static",
           "-Xcompiler", "-fPIC", "-Xlinker", "-soname=liblivre_gb300.so", "-lpthread", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    open(stamp, "w").write(dig)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force=True, verbose=True)
