"""Build libgbde.so (the C-ABI library) in-tree with nvcc for sm_103a.

Every translation unit under csrc/ is compiled in parallel with one
``-gencode arch=compute_103a,code=sm_103a`` and linked into
``libgbde.so`` next to this file.  Rebuilds only when a source is newer than
the library (or ``force=True``).
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libgbde.so")
OBJDIR = os.path.join(HERE, "_build")

NVCC_FLAGS = [
    "-std=c++17",
    "-O3",
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-lineinfo",
    "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
    "-Xptxas", "-warn-spills",
]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libgbde.so")


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


# Headers that runtime-compiled user models include (rtc.cu), embedded into
# the library as {include name, text}; gbde.h under the name models.cuh uses.
RTC_HEADERS = ["common.cuh", "controller.h", "solver.cuh", "models.cuh", "ff.cuh", "tableaus.h",
               "dense_coeffs.h", "explicit_rk.cuh", "rosenbrock.cuh", "ff_vec.cuh", "rodas_ff.cuh",
               "tsit5_ff.cuh", "vern7_ff.cuh", "ros23_ff.cuh", "dual.cuh", "philox.h", "sde.cuh",
               "autoswitch.cuh"]


def write_rtc_headers():
    """Write _build/rtc_headers.inc (only when its content changes)."""
    items = [(h, os.path.join(CSRC, h)) for h in RTC_HEADERS]
    items.append(("../../include/gbde.h", os.path.join(HERE, "..", "include", "gbde.h")))
    out = ["// generated by build.py from the library's headers; do not edit",
           "static const RtcHeader kRtcHeaders[] = {"]
    for name, path in items:
        text = open(path).read()
        if ")GBDE_RTC_\"" in text:
            raise RuntimeError("%s contains the raw-string delimiter" % name)
        out.append('  {"%s", R"GBDE_RTC_(%s)GBDE_RTC_"},' % (name, text))
    out.append("};")
    content = "\n".join(out) + "\n"
    path = os.path.join(OBJDIR, "rtc_headers.inc")
    if not os.path.exists(path) or open(path).read() != content:
        with open(path, "w") as f:
            f.write(content)


def _deps():
    return sources() + glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(
        os.path.join(CSRC, "*.cuh")) + [os.path.join(HERE, "..", "include", "gbde.h"), __file__]


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps() if os.path.exists(d))


def build(force=False, jobs=None, verbose=False):
    """Compile and link libgbde.so; returns its path."""
    if not force and up_to_date():
        return LIB
    nvcc = _nvcc()
    os.makedirs(OBJDIR, exist_ok=True)
    write_rtc_headers()
    srcs = sources()

    def compile_one(src):
        obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
        cmd = [nvcc] + NVCC_FLAGS + ["-I", OBJDIR, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        return obj

    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp"
    cmd = [nvcc, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", tmp] + objs + ["-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True))
