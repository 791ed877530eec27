"""The reference-arithmetic mode's kernels (GBODE_REF, compiled at run time
by NVRTC on a GPU host) also compile ahead of time for sm_103a with nvcc on a
machine without a GPU: an adaptive, a fixed-step and a Kuramoto kernel, so
that a change to the REF paths of ode_solver.cuh or crpow.h that does not
compile fails here, before any GPU run."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "simplediffeq.jl_gb300", "csrc")

TU = r'''
#define GBODE_BLOCK 128
#define GBODE_STAGE_BYTES 12288
#define GBODE_REF 1
#include "ode_solver.cuh"
typedef gbode::RhsLorenz<double, double> R0;
GBODE_ENTRY(ref_atsit5_plain, plain, gbode::MTsit5, gbode::PFP64, R0)
typedef gbode::RhsKuramoto<double, double, 3> R1;
GBODE_ENTRY(ref_kuramoto_plain, plain, gbode::MTsit5, gbode::PFP64, R1)
typedef gbode::RhsVanDerPol<double, double> R2;
GBODE_ENTRY(ref_rk4_onestep, onestep, gbode::MRK4, gbode::PFP64, R2)
'''


def test_reference_arithmetic_kernels_compile(tmp_path):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("nvcc not available")
    src = tmp_path / "ref_tu.cu"
    src.write_text(TU)
    r = subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "--fmad=false",
                        "-I", CSRC, "-c", str(src), "-o", str(tmp_path / "ref_tu.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
