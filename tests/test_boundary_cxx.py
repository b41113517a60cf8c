"""The compiled drop-in boundary: kodama_gb300/cxx/kodama_cuda_backend.cpp
built against the reference's own kodama.hpp and linked into the reference's
C++ core in place of its *_CUDA stubs (oracle/build_boundary.sh).

The driver (tests/boundary/boundary_driver.cpp) calls the reference's public
dispatching functions (KODAMAMatrix, KODAMAGraph, KODAMAMatrixFromGraph --
whose features the reference's own host code computes -- KNNCV, CoreKNN, CorePLSLDA,
PLSLDACV, PLSDACV, PLSLDAPredict; KODAMAMatrix on a host graph, which calls
CoreKNNGraph_CUDA per run; the CUDA proximity of KODAMADissimilarityInPlace)
with Backend::CUDA.  Compiling proves the shim matches the reference's
declarations and result structs field for field; on this host without a GPU
each call must end in the GB300 library's own "no CUDA device" error, which
proves the dispatch reached it and not the reference's "requires a CUDA
build" stub.  The CPU backend of the same binary still runs the reference.

The reference headers exist only where the reference checkout does, so this
check runs on the CPU host; the GPU host has no kodama.hpp to build it with."""

import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "oracle", "_ref", "boundary", "boundary_driver")

ENTRY_POINTS = ("KODAMAMatrix_CUDA", "KODAMAGraph_CUDA", "KODAMAMatrix(graph)->CoreKNNGraph_CUDA",
                "KODAMAMatrixFromGraphData_CUDA", "KODAMAMatrixFromGraph_CUDA", "KNNCV_CUDA", "CoreKNN_CUDA", "CorePLSLDA_CUDA", "PLSLDACV_CUDA",
                "PLSDACV_CUDA", "PLSLDAPredict_CUDA", "apply_kodama_dissimilarity_cuda")


@pytest.fixture(scope="module")
def driver_lines():
    from oracle import ref
    if not ref.available():
        pytest.skip("reference core (oracle/_ref) not built")
    from kodama_gb300 import build as kbuild
    kbuild.build()
    subprocess.run([os.path.join(ROOT, "oracle", "build_boundary.sh")], check=True)
    if not os.path.exists(DRIVER):
        pytest.skip("reference headers not present: the boundary driver was not built")
    import torch
    if torch.cuda.is_available():
        pytest.skip("this check expects a host without a GPU")
    out = subprocess.run([DRIVER], check=True, capture_output=True, text=True, timeout=600).stdout
    return dict(line.split("\t", 1) for line in out.strip().splitlines())


def test_cpu_backend_runs_the_reference(driver_lines):
    assert driver_lines["KODAMAMatrix[CPU]"] == "ok"


@pytest.mark.parametrize("name", ENTRY_POINTS)
def test_cuda_dispatch_reaches_the_library(driver_lines, name):
    msg = driver_lines[name]
    assert "requires a CUDA build" not in msg and "not enabled" not in msg, msg
    assert msg.startswith("kodama_gb300: ") and "no CUDA device" in msg, msg
