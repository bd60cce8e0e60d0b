"""Host-side pieces of bench.py that need no GPU: the command line, the
algorithmic-byte formula and the error report against the oracle."""
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_command_line_parses():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--help"], capture_output=True,
                         text=True, check=True).stdout
    for flag in ("--gpus", "--steps", "--warmup", "--impl", "--config"):
        assert flag in out


def test_algorithmic_bytes_formula():
    """B = 4 nnz_uu + 8 nnz_coupling + 8 rows + 8 (3 nu + 3 nu + n_p) + 8 n_mat
    for the mixed path, 8 nnz instead of the two Jacobian terms for FP64."""
    class Mesh:
        nu, n_pressure = 10, 3
        materials = np.zeros(2)

    class Set:
        ndofs, nnz, nnz_uu, nnz_coupling = 33, 500, 400, 100

    inputs = 8 * (30 + 30 + 3) + 16
    assert bench.algorithmic_bytes(Mesh, Set, True) == 4 * 400 + 8 * 100 + 8 * 33 + inputs
    assert bench.algorithmic_bytes(Mesh, Set, False) == 8 * 500 + 8 * 33 + inputs


def test_error_report_against_the_oracle():
    class FakeSet:  # 3 u rows (nu = 1) + 1 p row
        ndofs = 4

        class mesh:
            nu = 1

        @staticmethod
        def csr_pattern():
            return np.array([0, 5, 9, 13, 15]), None

        @staticmethod
        def mixed_layout():
            return np.array([0, 4, 7, 10]), np.array([0, 1, 2, 3, 5])

    rng = np.random.default_rng(0)
    vals = rng.normal(size=15)
    res = rng.normal(size=4)
    from cm_gb300.newton import mixed_positions
    uu_pos, cp_pos = mixed_positions(FakeSet)
    vu = vals[uu_pos].astype(np.float32)
    vc = vals[cp_pos].copy()
    vc[2] += 1e-9
    err = bench.error_vs_oracle(FakeSet, True, vu, vc, res + 1e-12, vals, res)
    assert err["residual"] <= 1e-12 / np.abs(res).max() * 1.01
    assert abs(err["coupling_blocks"] - 1e-9 / np.abs(vals[cp_pos]).max()) < 1e-15
    assert 0 < err["uu_block_fp32"] < 1e-6
    full = bench.error_vs_oracle(FakeSet, False, vals, None, res, vals, res)
    assert full["jacobian"] == 0.0 and full["residual"] == 0.0
