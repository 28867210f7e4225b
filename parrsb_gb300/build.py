"""Build the GB300 library: every .cu under csrc/ is compiled for sm_103a in
parallel and linked into parrsb_gb300/libparrsb_gb300.so (in-tree).

Flags: -fmad=false keeps every a*b+c an IEEE multiply and add (the bisection
keys must match the CPU restatement bit for bit); -lineinfo for profiling.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libparrsb_gb300.so")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC",
         "-Xcompiler", "-fvisibility=hidden", "--expt-relaxed-constexpr"]


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps():
    hdr = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    hdr.append(os.path.join(HERE, "..", "include", "parrsb.h"))
    return max(os.path.getmtime(h) for h in hdr)


def _compile(src, extra):
    obj = os.path.join(BUILD, src[:-3] + ".o")
    path = os.path.join(CSRC, src)
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(path), _deps()):
        return obj, None
    cmd = [NVCC] + ARCH + FLAGS + extra + ["-c", path, "-o", obj + ".tmp"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        # a failed compile is an error even when an older object exists
        if os.path.exists(obj):
            os.remove(obj)
        return obj, p.stdout + p.stderr
    os.replace(obj + ".tmp", obj)
    return obj, (p.stdout + p.stderr) if ("warning" in p.stderr.lower()) else None


def build(verbose=False, extra=()):
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    objs, errors = [], []
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        for obj, msg in ex.map(lambda s: _compile(s, list(extra)), srcs):
            objs.append(obj)
            if msg:
                (errors if not os.path.exists(obj) else []).append(msg)
                if verbose or not os.path.exists(obj):
                    sys.stderr.write(msg)
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lcudart"]
        subprocess.run(cmd, check=True)
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
