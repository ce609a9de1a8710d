"""Algorithmic byte models behind the roofline fractions bench.py reports,
pinned to the figures the committed ncu summaries use for the 64^3 hex8
workload (block nonzeros of an n^3 box: (3n+1)^3)."""
import os
import re

from tahoe_gb300 import workloads

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
N = 64
NND = (N + 1) ** 3
NEL = N ** 3
NNZB = (3 * N + 1) ** 3


def test_block_count_of_the_box():
    assert NNZB == 7_189_057 and NND == 274_625


def test_spmv_bytes_fp32():
    # nine FP32 values + column index per block, row pointers, p read, q written
    assert workloads.spmv_bytes(NNZB, NND, 4) == NNZB * 40 + (NND + 1) * 4 + 2 * NND * 16 == 297_448_784


def test_assembly_and_update_bytes_fp32():
    assert workloads.assembly_bytes(NEL, NNZB, NND, 4) == 856_185_208 + NND * 16  # + Jacobi's compact diagonal
    assert workloads.update_bytes(NND, 4) == NND * 164 == 45_038_500


def test_profiled_traffic_matches_the_byte_model():
    # the committed ncu summary of the product: DRAM traffic within 2 % of the model
    with open(os.path.join(ROOT, "profiles", "pcg_spmv_c2_64cubed.md")) as f:
        m = re.search(r"^traffic_bytes_per_launch: (\d+)$", f.read(), re.M)
    assert m, "summary carries the traffic line bench.py reads"
    traffic = int(m.group(1))
    assert abs(traffic / workloads.spmv_bytes(NNZB, NND, 4) - 1.0) < 0.02


def test_push_profile_traffic_matches_the_dram_model():
    # the push storage's product: DRAM traffic of the committed capture within
    # 1 % of the DRAM model (its pushed products stay in the L2 and are
    # counted apart)
    with open(os.path.join(ROOT, "profiles", "pcg_cg_push_c2_64cubed.md")) as f:
        m = re.search(r"^traffic_bytes_per_launch: (\d+)$", f.read(), re.M)
    assert m
    traffic = int(m.group(1))
    assert abs(traffic / workloads.spmv_bytes_push(NNZB, NND, 4) - 1.0) < 0.01
    nu, nl = (NNZB + NND) // 2, (NNZB - NND) // 2
    assert workloads.push_l2_bytes(NNZB, NND, 4) == nl * 16
    assert workloads.spmv_bytes_push(NNZB, NND, 4) == nu * 44 + (NND + 1) * 4 + 2 * NND * 16
