"""The drop-in boundary: the reference's solver templates compiled, unchanged, over the CUDA
backend of include/utopia_cuda_backend.hpp (CudaTraits, CuMatrix, CuVector).

tests/backend/cuda_backend_solvers.cpp instantiates ConjugateGradient + InvDiagPreconditioner,
Multigrid (Chebyshev3level / Jacobi / PointJacobi smoothing, IPRTransfer, Galerkin assembly,
dense Cholesky coarse solve) as a preconditioner and as a stand-alone solver, MPRGP and
ProjectedGaussSeidel.  It is built three times from the reference checkout's headers:

* over the oracle's CPU backend (oracle/ref/utopia_ref_backend.hpp);
* over the CUDA backend linked against tests/backend/fake_ugpu.cpp, a CPU stand-in of the C ABI
  with the same arithmetic order -- both runs must agree bit for bit, which checks the backend
  header's own logic (host mirrors and their offload flags, aliasing, the residual,
  triple-product and fused-dot specialisations);
* over the CUDA backend linked against libugpu.so -- the real drop-in; without a GPU it must
  report the missing device and exit 3.

CPU only; skipped where the reference checkout is not present (the GPU machine has none, so
the GPU run of this program is not part of the -m gpu tests).
"""
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ref = pytest.importorskip("oracle.ref")
if not ref.reference_available():
    pytest.skip("the reference checkout is not present", allow_module_level=True)

SRC = os.path.join(ROOT, "tests", "backend", "cuda_backend_solvers.cpp")
FAKE = os.path.join(ROOT, "tests", "backend", "fake_ugpu.cpp")
OUT = os.path.join(ROOT, "tests", "backend", "_build")


@pytest.fixture(scope="module")
def binaries():
    from utopia_gb300 import build

    ref.build_ref()
    lib = build.build()
    os.makedirs(OUT, exist_ok=True)
    inc = ref._include_flags(ref.DEFAULT_REFERENCE) + ["-I", os.path.join(ROOT, "include")]
    base = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-w"]
    support = sorted(os.path.join(ref._OUT, "obj", f) for f in os.listdir(os.path.join(ref._OUT, "obj"))
                     if f.startswith("utopia_"))

    def make(name, defines, extra_srcs, libs):
        exe = os.path.join(OUT, name)
        cmd = base + inc + defines + ["-o", exe, SRC] + extra_srcs + support + libs
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
        return exe

    libdir = os.path.dirname(lib)
    jobs = {
        "ref": ([], [], []),
        "cuda_fake": (["-DUSE_CUDA_BACKEND"], [FAKE], []),
        "cuda": (["-DUSE_CUDA_BACKEND"], [], ["-L" + libdir, "-lugpu", "-Wl,-rpath," + libdir, "-Wl,--no-undefined"]),
    }
    with ThreadPoolExecutor(3) as ex:
        futs = {k: ex.submit(make, "solvers_" + k, *v) for k, v in jobs.items()}
        return {k: f.result() for k, f in futs.items()}


def run(exe, n=32):
    return subprocess.run([exe, str(n)], capture_output=True, text=True, timeout=600)


def test_reference_templates_over_the_cuda_backend_match_the_cpu_backend(binaries):
    a, b = run(binaries["ref"]), run(binaries["cuda_fake"])
    assert a.returncode == 0, a.stderr
    assert b.returncode == 0, b.stderr
    lines_a, lines_b = a.stdout.split("\n"), b.stdout.split("\n")
    names = [line.split()[0] for line in lines_a if line]
    assert names == ["cg_invdiag", "mg_pcg_chebyshev", "mg_standalone", "mg_pcg_jacobi", "mg_pcg_point_jacobi",
                     "mprgp", "projected_gauss_seidel"]
    assert lines_a == lines_b  # iterations, reasons, ||x|| and sum(x) to 17 digits
    for line in lines_a:
        if line:
            name, its, reason = line.split()[:3]
            assert int(reason) > 0 or name == "mg_standalone", line


def test_cuda_backend_links_against_libugpu_and_reports_a_missing_device(binaries):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = run(binaries["cuda"])
    assert r.returncode == 3
    assert "no device" in r.stderr
