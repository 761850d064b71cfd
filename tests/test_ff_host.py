"""The float-float arithmetic of the FP32-bulk residual (ff.cuh), on the
host: sums (including nearly cancelling ones), products, quotients and square
roots of seeded operands over 24 decades against long double.  Bound: 2^-44
(5.7e-14) relative, against the 2^-24 (6e-8) of plain FP32.  The bit-level
conversions (ff_split: double -> float-float to 2^-47 and normalised;
ff_widen: float -> double bit for bit; ff_to_double_bits) on the same
operands.  The float-float matvec's row sums (ff_axpy over 324 terms of
float K and split double x): 2^-44 relative to sum |K x|."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_float_float_operations_hold_48_bits(tmp_path):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if Path("/usr/local/cuda/bin/nvcc").exists() else None)
    if nvcc is None:
        pytest.skip("nvcc not available")
    exe = tmp_path / "ff_host"
    subprocess.run([nvcc, "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a",
                    str(ROOT / "tests" / "ff_host.cu"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    e_add, e_cancel, e_mul, e_div, e_sqrt, e_split = map(float, out[:6])
    bad_norm, bad_widen, bad_todouble, zeros = map(int, out[6:10])
    e_dot = float(out[10])
    bound = 2.0 ** -44
    assert e_add <= bound and e_cancel <= bound, (e_add, e_cancel)
    assert e_mul <= bound and e_div <= bound and e_sqrt <= bound, (e_mul, e_div, e_sqrt)
    # the bit-level conversions of the residual kernel's inputs and outputs
    assert e_split <= 2.0 ** -47, e_split
    assert bad_norm == 0 and bad_widen == 0 and bad_todouble == 0 and zeros == 1, out
    assert e_dot <= bound, e_dot
