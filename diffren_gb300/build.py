"""Builds libdiffren_gb300.so in-tree with nvcc for sm_103a.

Each .cu file compiles to an object in parallel, then nvcc links the shared
library against the shared CUDA runtime (the one torch already loaded), with
an rpath to the toolkit for use without torch.
"""
import concurrent.futures
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libdiffren_gb300.so")
SOURCES = ["raster.cu", "interp.cu", "splat.cu", "texture.cu", "normals.cu", "composite.cu",
           "loss.cu", "light.cu", "abi.cu", "static_scratch.cu"]
HEADERS = ["common.cuh", "internal.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
  cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
  path = os.path.join(cuda, "bin", "nvcc")
  return path if os.path.exists(path) else "nvcc"


def _flags():
  return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                 "-Xcompiler", "-O2", "-I", os.path.join(ROOT, "include"),
                 "-I", CSRC]


def _stale(target, deps):
  if not os.path.exists(target):
    return True
  t = os.path.getmtime(target)
  return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra_flags=()):
  """Compiles (if needed) and returns the path of libdiffren_gb300.so."""
  os.makedirs(BUILD, exist_ok=True)
  headers = [os.path.join(CSRC, h) for h in HEADERS]
  headers.append(os.path.join(ROOT, "include", "diffren_gb300.h"))
  jobs = []
  objs = []
  for src in SOURCES:
    s = os.path.join(CSRC, src)
    o = os.path.join(BUILD, src.replace(".cu", ".o"))
    objs.append(o)
    if force or _stale(o, [s] + headers):
      jobs.append([nvcc()] + _flags() + list(extra_flags) + ["-c", s, "-o", o])

  def run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
      raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    if verbose and (r.stdout or r.stderr):
      sys.stderr.write(r.stdout + r.stderr)

  if jobs:
    with concurrent.futures.ThreadPoolExecutor(len(jobs)) as ex:
      list(ex.map(run, jobs))
  if force or jobs or _stale(LIB, objs):
    cuda = os.path.dirname(os.path.dirname(nvcc())) if os.path.isabs(nvcc()) else "/usr/local/cuda"
    run([nvcc()] + ARCH + ["-shared", "-cudart", "shared", "-o", LIB] + objs +
        ["-Xlinker", "-rpath," + os.path.join(cuda, "lib64")])
  return LIB


if __name__ == "__main__":
  print(build(force="--force" in sys.argv, verbose=True,
              extra_flags=["-Xptxas", "-v"] if "--ptxas" in sys.argv else []))
