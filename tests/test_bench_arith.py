"""The roofline arithmetic of bench.py, pinned on the benchmark workload
(3-D 7-point Laplacian 128^3, Lanczos m = 80): per step the SpMV reads the
values and column indices (12 B per stored entry), the row pointers (4 B per
row + 1) and v_i, and writes u (16 B per row); the three-term update reads
u, v_i and v_{i-1} and writes v_{i+1} (32 B per row); step 1 has no v_{i-1}.
CPU only."""
import bench
from psfun_gb300 import matrices

N, NNZ = 2_097_152, 14_581_760


def test_workload_sizes():
    A = matrices.laplacian_3d(128)
    assert (A.shape[0], A.nnz) == (N, NNZ)
    assert "n=2,097,152" in bench.WORKLOAD and "nnz=14,581,760" in bench.WORKLOAD
    assert bench.M_KRYLOV == 80 and bench.T_EXP == 0.05


def test_bytes_per_step_and_launch():
    b = bench.algorithmic_bytes(N, NNZ)
    assert b["spmv"] == 12 * NNZ + 4 * (N + 1) + 16 * N == 216_924_164
    assert b["update"] == 32 * N
    assert b["step"] == 284_033_028
    assert bench.persist_bytes(N, NNZ, 80) == 80 * 284_033_028 - 8 * N == 22_705_865_024
