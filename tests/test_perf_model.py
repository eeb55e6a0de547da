"""The algorithmic cost model (spectrax_gb300/perf.py) on the plan's radices (no GPU)."""
from spectrax_gb300 import perf


def test_step_vectors():
    assert perf.dopri8_vectors_per_step_dense(13) == 120
    assert perf.dopri8_vectors_per_step() <= 120


def test_rhs_ops_follow_the_product_grid_radices():
    # the two-stream shape, 6-plane tiles, packed: the 144-point grid of radices
    # 4*4*3*3 needs fewer FP64 instructions than the 129-point 43*3 transforms
    shape = (129, 1, 1, 256, 1, 1, 3)
    nx = perf.rhs_ops(shape, 6, 43, None, packed=True)
    m144 = perf.rhs_ops(shape, 6, 43, 144, packed=True, radices=(4, 4, 3, 3))
    assert 0.0 < m144.instr < nx.instr
    # radices given explicitly are used as given: a worse order costs more
    m144b = perf.rhs_ops(shape, 6, 43, 144, packed=True, radices=(8, 2, 3, 3))
    assert m144b.instr != m144.instr
    # flops count an FMA twice
    assert m144.flops > m144.instr


def test_fft_line_ops_register_radices():
    # one 16-point line of radices 4*4: 4 radix-4 butterflies (16 FP64 each), then
    # 3 twiddled butterflies (3 complex multiplies each, 4 instructions) + 4 butterflies
    o = perf.fft_line_ops(16, None, "dit", [4, 4])
    assert o.instr == 4 * 16 + 3 * 3 * 4 + 4 * 16
