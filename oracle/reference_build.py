"""Recipe that compiles pieces of the reference from their own sources, in
place, into oracle/_ref/ (TEST INFRASTRUCTURE ONLY; outputs are not
committed).

Built here:
  * contact_geometry_tests -- the reference's own known-answer test
    (tests/contact_geometry_test.cpp + src/contact_geometry.cpp);
  * libref_geometry.so -- the reference's CPU sphere/triangle overlap area
    (src/contact_geometry.cpp) behind oracle/ref_geometry_harness.cpp.
The reference's CUDA step engine itself needs a GPU and its CMake build; it
is not built here.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")


def build(ref_root="/root/reference"):
    if not os.path.isdir(ref_root):
        return None
    os.makedirs(OUT, exist_ok=True)
    inc = os.path.join(ref_root, "include")
    geo = os.path.join(ref_root, "src", "contact_geometry.cpp")
    test = os.path.join(ref_root, "tests", "contact_geometry_test.cpp")
    flags = ["-O2", "-std=c++17", "-ffp-contract=off", "-I", inc]
    subprocess.run(["g++", *flags, "-o", os.path.join(OUT, "contact_geometry_tests"), test, geo], check=True)
    subprocess.run(["g++", *flags, "-shared", "-fPIC", "-o", os.path.join(OUT, "libref_geometry.so"),
                    os.path.join(HERE, "ref_geometry_harness.cpp"), geo], check=True)
    return OUT


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else "/root/reference"))
