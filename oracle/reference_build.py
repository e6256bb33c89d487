"""Recipe that compiles pieces of the reference from their own sources, in
place, into oracle/_ref/ (TEST INFRASTRUCTURE ONLY; outputs are not
committed).

The reference tree is found through DEM_REFERENCE_ROOT; this recipe is the
one place that also knows the reference's checkout path in the build
container (REFERENCE_DEFAULT), which is used when the variable is unset.

Built here:
  * contact_geometry_tests -- the reference's own known-answer test
    (tests/contact_geometry_test.cpp + src/contact_geometry.cpp);
  * libref_geometry.so -- the reference's CPU sphere/triangle overlap area
    (src/contact_geometry.cpp) behind oracle/ref_geometry_harness.cpp;
  * ref_engine.cubin -- the device code of the reference's CUDA engine
    (src/cuda/cuda_{particle,grid,body,contact}_backend.cu) for sm_103a,
    compiled the way the reference's CMakeLists.txt:39-55 builds it: C++17,
    -O3, DEM_MBD_USE_CUDA=1, separable compilation (-rdc=true) and a device
    link.  Device code needs no host compiler of the target machine, so the
    same file runs on the Arm GPU hosts; oracle/ref_cuda_host.cu launches it
    there.  ref_engine_kernels.json maps each kernel's short name to the
    entry name ptxas reports (-Xptxas -v);
  * ref_layout_check -- compiled from the reference's headers and
    oracle/ref_cuda_layout.h; it fails to compile unless every device
    structure restated in ref_cuda_layout.h has the reference's size and
    field offsets, so the launcher passes kernel arguments byte for byte.
"""
import json
import os
import re
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REFERENCE_DEFAULT = "/root/reference"
CUBIN = os.path.join(OUT, "ref_engine.cubin")
KERNELS = os.path.join(OUT, "ref_engine_kernels.json")
CUDA_UNITS = ["cuda_particle_backend", "cuda_grid_backend", "cuda_body_backend", "cuda_contact_backend"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def reference_root():
    """The reference checkout, or None when it is not present on this machine."""
    root = os.environ.get("DEM_REFERENCE_ROOT", REFERENCE_DEFAULT)
    return root if os.path.isdir(os.path.join(root, "src", "cuda")) else None


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _short_name(unit, mangled):
    """'particle.advancePositionKernel' from a mangled entry name: the name is
    the identifier ending in 'Kernel' whose decimal length prefix matches it."""
    for m in re.finditer(r"(?=(\d+)([A-Za-z_]\w*?Kernel)E)", mangled):
        digits, name = m.group(1), m.group(2)
        if any(int(digits[k:]) == len(name) for k in range(len(digits))):
            return unit.replace("cuda_", "").replace("_backend", "") + "." + name
    return None


def build_cuda(ref_root):
    """Reference device code -> oracle/_ref/ref_engine.cubin (+ kernel name map)."""
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    inc = ["-I", os.path.join(ref_root, "include"), "-I", os.path.join(ref_root, "src")]
    objs = {}

    def one(unit):
        src = os.path.join(ref_root, "src", "cuda", unit + ".cu")
        obj = os.path.join(OUT, unit + ".rdc.cubin")
        cmd = [nvcc, *ARCH, "-rdc=true", "-cubin", "-O3", "-std=c++17", "-DDEM_MBD_USE_CUDA=1", *inc,
               "-Xptxas", "-v", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s" % (unit, r.stderr))
        names = re.findall(r"Compiling entry function '([^']+)'", r.stderr)
        return unit, obj, names

    with ThreadPoolExecutor(len(CUDA_UNITS)) as ex:
        results = list(ex.map(one, CUDA_UNITS))
    table = {}
    for unit, obj, names in results:
        objs[unit] = obj
        for mangled in names:
            short = _short_name(unit, mangled)
            if short is not None and "GLOBAL__N" in mangled:
                table[short] = mangled
    tmp = CUBIN + ".tmp"
    cmd = [nvcc, *ARCH, "-dlink", "-cubin", *[objs[u] for u in CUDA_UNITS], "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("device link failed:\n" + r.stderr)
    os.replace(tmp, CUBIN)
    for unit in CUDA_UNITS:
        os.remove(objs[unit])
    with open(KERNELS, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    return CUBIN


def check_layout(ref_root):
    """Compile oracle/ref_layout_check.cpp against the reference's headers."""
    os.makedirs(OUT, exist_ok=True)
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-I", "/usr/local/cuda/include",
           "-I", os.path.join(ref_root, "src", "cuda"), "-I", HERE, os.path.join(HERE, "ref_layout_check.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("restated reference layouts differ from the reference's headers:\n" + r.stderr)
    with open(os.path.join(OUT, "ref_layout_check.ok"), "w") as f:
        f.write("ok\n")


def build(ref_root=None):
    ref_root = ref_root or reference_root()
    if ref_root is None or not os.path.isdir(ref_root):
        return None
    os.makedirs(OUT, exist_ok=True)
    inc = os.path.join(ref_root, "include")
    geo = os.path.join(ref_root, "src", "contact_geometry.cpp")
    test = os.path.join(ref_root, "tests", "contact_geometry_test.cpp")
    flags = ["-O2", "-std=c++17", "-ffp-contract=off", "-I", inc]
    subprocess.run(["g++", *flags, "-o", os.path.join(OUT, "contact_geometry_tests"), test, geo], check=True)
    subprocess.run(["g++", *flags, "-shared", "-fPIC", "-o", os.path.join(OUT, "libref_geometry.so"),
                    os.path.join(HERE, "ref_geometry_harness.cpp"), geo], check=True)
    if os.path.exists(os.path.join(HERE, "ref_layout_check.cpp")):
        check_layout(ref_root)
    build_cuda(ref_root)
    return OUT


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else None))
