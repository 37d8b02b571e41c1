"""Build helper for the C++ API test program (tests/cpp/nscale_api_test.cpp)."""
import os
import shutil
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "emory-cci-fast-ia-gsoc_gb300", "lib")
SRC = os.path.join(ROOT, "tests", "cpp", "nscale_api_test.cpp")


def cuda_home():
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return "/usr/local/cuda"


def build(out_path):
    cuda = cuda_home()
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-I", os.path.join(ROOT, "include"), "-I",
           os.path.join(cuda, "include"), SRC, "-o", out_path, "-L", LIBDIR, "-lnsgb",
           "-L", os.path.join(cuda, "lib64"), "-lcudart", "-Wl,-rpath," + LIBDIR,
           "-Wl,-rpath," + os.path.join(cuda, "lib64")]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
