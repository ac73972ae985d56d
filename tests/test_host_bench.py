"""Host-side pieces of bench.py (no GPU): the algorithmic-bytes formula of
the headline workload, the traffic figures read from the committed ncu
summaries, and the kernel names each --kernel choice reports."""
import bench


def test_algorithmic_bytes_of_the_headline_workload():
    # 64^3 x 6 tets: 1,572,864 cells, 274,625 points, nnz 36,200,448, 4,743,168 DoF
    T, V, nnz, n_dof = 6 * 64 ** 3, 65 ** 3, 36_200_448, 4_743_168
    fp32 = bench.algorithmic_bytes(T, V, nnz, n_dof, 4)
    # vertex ids + coordinates + kappa and f + orientation byte + values + residual
    assert fp32 == T * 16 + V * 24 + 2 * T * 4 + T + nnz * 4 + n_dof * 4 == 209_687_064
    assert bench.algorithmic_bytes(T, V, nnz, n_dof, 8) - fp32 == 2 * T * 4 + nnz * 4 + n_dof * 4
    # triangles carry three vertex ids per cell
    assert bench.algorithmic_bytes(10, 8, 40, 25, 4, verts_per_cell=3) == 10 * 12 + 8 * 24 + 80 + 10 + 160 + 100


def test_profiled_traffic_is_read_from_the_summaries():
    assert bench.profiled_traffic("darcy_records_rows_f32_cube64.txt") == 305_379_840
    assert bench.profiled_traffic("darcy_rows_f32_cube64.txt") == 314_387_200
    assert bench.profiled_traffic("elasticity_rows_f32_cube40.txt") == 711_353_344
    assert bench.profiled_traffic("darcy_records_rows_f64_cube64.txt") == 625_029_632
    assert bench.profiled_traffic("darcy_records_rows_f32_batch512.txt") == 1_143_034_624
    assert bench.profiled_traffic("no_such_summary.txt") is None


def test_job_rate_counts_every_rank():
    assert bench.job_rate(1000, 4, 2.0) == 4 * 1000 / 2e-3
