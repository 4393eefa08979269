"""Build libtisphi_gb300.so for sm_103a with nvcc (no CMake, no torch extension).

Each translation unit compiles in parallel; units whose results must round exactly like
the f64 oracle (the sort and the FP64 form) get -fmad=false so that no multiply-add is
contracted into an FMA.  Outputs: tisphi_gb300/_build/*.o and tisphi_gb300/libtisphi_gb300.so.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libtisphi_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--extended-lambda",
          "--expt-relaxed-constexpr", "-I", INCLUDE, "-Xptxas", "-warn-spills"]
UNITS = {
    "tsg_api.cu": ["-fmad=false"],
    "tsg_sort.cu": ["-fmad=false"],
    "tsg_fp64.cu": ["-fmad=false"],
    "tsg_fp32.cu": [],
    "tsg_adjoint.cu": [],
    "tsg_visual.cu": ["-fmad=false"],
    "tsg_noalloc.cu": ["-fmad=false"],
}


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _deps():
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hdrs.append(os.path.join(INCLUDE, "tisphi_gb300.h"))
    return max(os.path.getmtime(h) for h in hdrs)


def _compile(src, extra, hdr_time, verbose):
    obj = os.path.join(BUILD, src.replace(".cu", ".o"))
    path = os.path.join(CSRC, src)
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(path), hdr_time):
        return obj, ""
    cmd = [_nvcc()] + ARCH + COMMON + extra + ["-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, (r.stdout + r.stderr) if verbose else ""


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    hdr_time = _deps()
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        futs = [ex.submit(_compile, s, e, hdr_time, verbose) for s, e in UNITS.items()]
        objs = []
        for f in futs:
            obj, log = f.result()
            objs.append(obj)
            if log:
                print(log, file=sys.stderr)
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs):
        return LIB
    cmd = [_nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
