"""Builds libdegpu.so in place: every CUDA translation unit for sm_103a, in parallel; and
libdegpu_probe.so from probe/ (the FMA peak probe and device self-checks used by the benchmark and
the tests, kept out of the integrator library).

Usage: python build.py [--jobs N] [--verbose]
The parity translation units (inst_parity_*.cu) and the shooting Newton kernels (bvp.cu) are
compiled with -fmad=false so that no multiply-add on those paths is contracted into an FMA.
"""
import argparse
import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "libdegpu.so")
PROBE_OUT = os.path.join(HERE, "libdegpu_probe.so")
BUILD = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no multiply-add contraction (gcc contracts by default on aarch64), so host-side FP64
# arithmetic such as the hyperplane normal's scaling rounds as the crate's does
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
          "-Xcompiler", "-ffp-contract=off",
          "-diag-suppress", "20091", "-I", os.path.join(HERE, "..", "..", "include")]
PARITY = ["-fmad=false", "-DDEGPU_NO_FMAD"]


def nvcc():
    import shutil
    found = shutil.which("nvcc")
    if found:
        return found
    for root in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if root and os.path.exists(os.path.join(root, "bin", "nvcc")):
            return os.path.join(root, "bin", "nvcc")
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(glob.glob(os.path.join(HERE, "*.cu")))


def flags_for(src):
    name = os.path.basename(src)
    f = list(ARCH) + list(COMMON)
    # extra nvcc flags for tuning experiments, e.g. DEGPU_NVCC_EXTRA="-DDEGPU_MIXED_MIN_BLOCKS=8"
    f += os.environ.get("DEGPU_NVCC_EXTRA", "").split()
    # the parity kernels, and the shooting Newton kernels (bvp.cu), which restate the crate's
    # arithmetic on the device
    if name.startswith("inst_parity") or name == "bvp.cu":
        f += PARITY
    return f


def needs(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + glob.glob(os.path.join(HERE, "*.cuh")) + glob.glob(os.path.join(HERE, "*.inc")) + \
        glob.glob(os.path.join(HERE, "..", "..", "include", "*.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def compile_one(src, verbose):
    probe = os.path.basename(os.path.dirname(src)) == "probe"
    obj = os.path.join(BUILD, ("probe_" if probe else "") + os.path.basename(src) + ".o")
    if not needs(obj, src):
        return obj, ""
    cmd = [nvcc()] + flags_for(src) + (["-I", HERE] if probe else []) + ["-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(jobs=None, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    probe_srcs = sorted(glob.glob(os.path.join(HERE, "probe", "*.cu")))
    jobs = jobs or min(len(srcs) + len(probe_srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        futs = [ex.submit(compile_one, s, verbose) for s in srcs]
        probe_futs = [ex.submit(compile_one, s, verbose) for s in probe_srcs]
        objs = [f.result()[0] for f in futs]
        probe_objs = [f.result()[0] for f in probe_futs]
    for out, os_, libs in ((OUT, objs, ["-lcudart", "-lnvrtc"]), (PROBE_OUT, probe_objs, ["-lcudart"])):
        if not os.path.exists(out) or any(os.path.getmtime(o) > os.path.getmtime(out) for o in os_):
            cmd = [nvcc()] + ARCH + ["-shared", "-o", out] + os_ + libs
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return OUT


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=None)
    ap.add_argument("--verbose", action="store_true")
    args = ap.parse_args()
    print(build(args.jobs, args.verbose))
