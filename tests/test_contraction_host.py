"""The element contraction K_e = N^T D N of the row assembly (row_w_entry,
row_block_entry and skew_entry in element.cuh), run on the host for every
patch size 1-step subdivision gives (nen = 10..16, including the ones no test
mesh reaches on the device), with and without the follower-pressure blocks,
against numpy.  Every entry must be written."""
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
NVCC = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if Path("/usr/local/cuda/bin/nvcc").exists() else None)


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    if NVCC is None:
        pytest.skip("nvcc not available")
    exe = tmp_path_factory.mktemp("contract") / "contract_host"
    subprocess.run([NVCC, "-std=c++17", "--expt-relaxed-constexpr", "-O2",
                    "-gencode", "arch=compute_103a,code=sm_103a",
                    str(ROOT / "tests" / "contract_host.cu"), "-o", str(exe)], check=True)
    return exe


def reference(D, N, nen, cslot, pres, vv, sc):
    """K[(a,i),(b,j)] = sum_{r,s} N[r][a] D[3r+i][3s+j] N[s][b] plus, for corner
    rows a and corner column b = cslot[k], the cross-product matrix of sc vv[k]."""
    Nx = np.kron(N[:, :nen], np.eye(3))            # (15, 3 nen)
    K = Nx.T @ D @ Nx                               # (3 nen, 3 nen), rows (a,i), cols (b,j)
    if pres:
        for k in range(3):
            v = sc * vv[k]
            skew = np.array([[0, -v[2], v[1]], [v[2], 0, -v[0]], [-v[1], v[0], 0]])
            b = cslot[k]
            for a in cslot:
                K[3 * a:3 * a + 3, 3 * b:3 * b + 3] += skew
    # block layout (a nen + b) 9 + 3i + j
    return K.reshape(nen, 3, nen, 3).transpose(0, 2, 1, 3).reshape(-1)


@pytest.mark.parametrize("nen", [10, 11, 12, 13, 14, 15, 16])
@pytest.mark.parametrize("pres", [False, True])
def test_contraction_matches_numpy(driver, tmp_path, nen, pres):
    rng = np.random.default_rng(1000 + 2 * nen + pres)
    D = rng.standard_normal((15, 15))
    N = np.zeros((5, 16))
    N[:, :nen] = rng.standard_normal((5, nen))
    cslot = rng.choice(nen, 3, replace=False).astype(np.int32)
    vv = rng.standard_normal((3, 3))
    sc = -1e-3 / 6
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as f:
        f.write(np.array([nen, *cslot, int(pres)], np.int32).tobytes())
        f.write(D.astype(np.float64).tobytes())
        f.write(N.astype(np.float64).tobytes())
        f.write(vv.astype(np.float64).tobytes())
        f.write(np.array([sc]).tobytes())
    subprocess.run([str(driver), str(inp), str(out)], check=True)
    res = np.fromfile(out, np.float64)
    n = 9 * nen * nen
    k64, k32 = res[:n], res[n:]
    assert np.isfinite(k64).all() and np.isfinite(k32).all()   # every entry written
    ref = reference(D, N, nen, cslot, pres, vv, sc)
    scale = np.abs(ref).max()
    np.testing.assert_allclose(k64, ref, rtol=0, atol=1e-13 * scale)
    np.testing.assert_allclose(k32, ref, rtol=0, atol=2e-5 * scale)
