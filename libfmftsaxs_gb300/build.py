"""Build the in-tree shared library libfmftsaxs_gb300.so (sm_103a kernels +
C11 host code) with nvcc and gcc.  No cmake; translation units compile in
parallel.  Kernels whose rounding must follow the reference are compiled
with -fmad=false; host C with -std=c11 -ffp-contract=off."""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfmftsaxs_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU = {"kernels_faithful.cu": ["-fmad=false"], "kernels_contract.cu": [], "kernels_lbfgsb.cu": ["-fmad=false"],
      "kernels_fitdf.cu": ["-fmad=false"], "kernels_tc.cu": [], "kernels_topk.cu": [],
      "kernels_ingest.cu": ["-fmad=false"]}
C = ["sxs_host.c", "sxs_api.c", "sxs_tables.c", "sxs_serve.c", "sxs_exact.c", "sxs_batch.c"]


def _cuda_home():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def build(verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
    jobs = []
    objs = []
    for src, extra in CU.items():
        o = os.path.join(OBJ, src + ".o")
        cmd = [nvcc] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-c",
                                os.path.join(CSRC, src), "-o", o] + extra + inc
        jobs.append(cmd)
        objs.append(o)
    for src in C:
        o = os.path.join(OBJ, src + ".o")
        cmd = ["gcc", "-std=c11", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
               "-I" + os.path.join(cuda, "include"), "-c", os.path.join(CSRC, src), "-o", o] + inc
        jobs.append(cmd)
        objs.append(o)
    procs = [(subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT), c) for c in jobs]
    failed = False
    for p, c in procs:
        out, _ = p.communicate()
        if verbose or p.returncode:
            sys.stderr.write(" ".join(c) + "\n" + out.decode(errors="replace"))
        failed |= p.returncode != 0
    if failed:
        raise RuntimeError("libfmftsaxs_gb300: compilation failed")
    link = [nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread", "-lm"]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode:
        sys.stderr.write(" ".join(link) + "\n" + r.stdout.decode(errors="replace"))
        raise RuntimeError("libfmftsaxs_gb300: link failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
