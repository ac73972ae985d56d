"""The double-float routines of the FP64 assembly (nfempy_gb300/csrc/df64.cuh)
compiled for the host with g++ and checked against long double: FP64 ->
double-float split within 2^-48, 64-bit fixed-point integers within
2^-47, the packing back to FP64 to half an ulp,
add / multiply / reciprocal / 3-term dot products within 2^-44 (operand
splits included); for the lattice records, the 64-bit fixed-point factor
within 2^-60, integer x fixed-point products packed into FP64 within one
ulp (2^-52), the scaled packing to half an ulp and 32-bit integers to
FP64 exactly.  No GPU needed."""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_df64_routines_against_long_double():
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "df64_check")
        subprocess.run([gxx, "-O2", "-std=c++17", "-o", exe, os.path.join(HERE, "native", "df64_check.cpp")],
                       check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    err = {k: float(v) for k, v in (line.split() for line in out.strip().splitlines())}
    assert err["split"] <= 2.0 ** -48 and err["i64"] <= 2.0 ** -47
    assert err["round"] <= 2.0 ** -53 and err["pack"] <= 2.0 ** -53
    assert err["q64"] <= 2.0 ** -60 and err["prod"] <= 2.0 ** -52 and err["scaled"] <= 2.0 ** -53
    assert err["i32"] == 0  # 32-bit integers to FP64 by bits, exactly
    for k in ("add", "mul", "recip", "dot"):
        assert err[k] <= 2.0 ** -44, (k, err[k])
