"""Build libddd_gb300.so in-tree with nvcc for sm_103a (GB300).

Each translation unit compiles in parallel into _build/, then one nvcc -shared
link.  No cmake, no torch extension machinery: the library exports a plain C
ABI (include/ddd_gb300.h).
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libddd_gb300.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]


# Translation units compiled more than once: (object suffix, extra flags).
VARIANTS = {
    "segseg_f64.cu": [("strict", ["-DDDD_VARIANT=strict", "--fmad=false"]), ("fast", ["-DDDD_VARIANT=fast"])],
    "sigma_f64.cu": [("strict", ["-DDDD_VARIANT=strict", "--fmad=false"]), ("fast", ["-DDDD_VARIANT=fast"])],
    # df64 needs exact error-free transformations: no contraction.
    "segseg_df.cu": [("", ["--fmad=false"])],
    # explicit fused multiply-adds only (host builds of its header give the same bits)
    "segseg_f64fast.cu": [("", ["--fmad=false"])],
    "sigma_fx.cu": [("", ["--fmad=false"])],
    "segseg_batch.cu": [("", ["--fmad=false"])],
    "surrogate_data.cu": [("", ["--fmad=false"])],
    "surrogate_force.cu": [("", ["--fmad=false"])],
    "self_force.cu": [("", ["--fmad=false"])],
    "mobility.cu": [("", ["--fmad=false"])],
    "collision.cu": [("", ["--fmad=false"])],
    "u_tilde.cu": [("", ["--fmad=false", "-Xcompiler", "-ffp-contract=off"])],
    "u_tilde_fast.cu": [("", ["--fmad=false"])],
}


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def units():
    """(source, object, extra flags) for every object of the library."""
    out = []
    for src in sources():
        base = os.path.basename(src)[:-3]
        for suffix, flags in VARIANTS.get(os.path.basename(src), [("", [])]):
            obj = os.path.join(BUILD, base + ("_" + suffix if suffix else "") + ".o")
            out.append((src, obj, flags))
    return out


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(HERE, "..", "include", "ddd_gb300.h"))
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, obj, extra, verbose):
    if not _stale(obj, [src] + _headers() + [__file__]):
        return obj, ""
    cmd = [NVCC] + ARCH + FLAGS + extra + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return obj, r.stderr if verbose else ""


def build(verbose=False, ptxas_info=False):
    os.makedirs(BUILD, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    us = units()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(us))) as ex:
        results = list(ex.map(lambda u: _compile(u[0], u[1], u[2] + extra, verbose or ptxas_info), us))
    objs = [o for o, _ in results]
    logs = "".join(l for _, l in results)
    if _stale(LIB, objs):
        tmp = LIB + ".tmp"
        cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
        os.replace(tmp, LIB)
    if logs:
        sys.stderr.write(logs)
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="-v" in sys.argv)
    print(LIB)
