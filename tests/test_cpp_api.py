"""The C++ library API (include/sl3dgpu.hpp, namespace sl3dpp): compiled with
g++ -std=c++23 against the library and the oracle, the way a C++ caller of
the reference builds against its headers.

The host half (argument checks, the error mapping to std::invalid_argument /
std::runtime_error, the load callables' layout) runs without a GPU; the GPU
half checks the band solvers, DegreeOperator / ToroidalOperator, three
Sdirk2 steps of Viscoelastic3D (delta given as a callable, loads as
LoadCallable3D) and one ElasticPerturbation3D::SolveLateral against the
oracle on the same inputs, a driver's own iteration through
Viscoelastic3D::OpenStep against the operator's step (bit for bit), the
GridCoupling maps' identities, ElasticPerturbation3D's Force / Apply /
LoadForces, GRDSolver's identities (generalised and nonlinear) and
Evolution3D's migrating run under still ice against its frozen run
(tests/cpp/test_api.cpp)."""

import pathlib
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
SOURCE = ROOT / "tests" / "cpp" / "test_api.cpp"
BINARY = ROOT / "tests" / "cpp" / "_build" / "test_api"


@pytest.fixture(scope="module")
def binary():
    import __graft_entry__
    from oracle import build as oracle_build
    from sl3dpp_gb300 import _lib

    __graft_entry__.build()
    oracle = oracle_build.build()
    BINARY.parent.mkdir(exist_ok=True)
    cmd = ["g++", "-std=c++23", "-O1", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"), str(SOURCE),
           "-o", str(BINARY),
           str(_lib.LIBRARY_PATH), f"-Wl,-rpath,{_lib.LIBRARY_PATH.parent}",
           str(oracle), f"-Wl,-rpath,{oracle.parent}", "-fopenmp"]
    result = subprocess.run(cmd, capture_output=True, text=True)
    assert result.returncode == 0, " ".join(cmd) + "\n" + result.stderr
    return BINARY


def _run(binary, mode, timeout):
    result = subprocess.run([str(binary), mode], capture_output=True, text=True, timeout=timeout)
    print(result.stdout)
    assert result.returncode == 0, result.stdout + result.stderr
    assert "FAIL" not in result.stdout
    return result.stdout


def test_header_compiles_as_cxx23_and_maps_errors_without_a_gpu(binary):
    out = _run(binary, "host", 120)
    assert "0 failures" in out


@pytest.mark.gpu
def test_cpp_api_matches_the_oracle_on_the_gpu(gpu, binary):
    out = _run(binary, "gpu", 900)
    assert "SolveLateral surface 2 matches the oracle" in out and "step 2 surface phi matches" in out
    assert "open step 1 surface 2 is the operator's step bit for bit" in out
    assert "ElasticPerturbation3D Force is linear" in out
    assert "GRDSolver SolveNonlinear without a moving shoreline is the linear solve" in out
    assert "Evolution3D RunMigrating under still ice is RunOcean's frozen run" in out
