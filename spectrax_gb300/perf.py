"""Algorithmic cost model of the GPU path (bytes and FP64 operations).

Bytes follow the definition "read every input vector once, write every output
vector once" (16 B per complex128 entry).  FP64 operations count the double
instructions the kernels issue (an FMA counts as 2 flops), from the FFT plan
(radices and spans) and the fused epilogues; they are checked against ncu's
SASS counters in ``profiles/``.
"""
from __future__ import annotations

from dataclasses import dataclass

def dopri8_vectors_per_step_dense(s: int = 13) -> int:
    """Vectors per step of an s-stage method whose stage i reads y and all i - 1
    earlier K_j and writes K_i, whose last combination reads s + 1 vectors and
    writes y_new and the error: s (s + 3) / 2 + s + 3 (120 for s = 13)."""
    return s * (s + 3) // 2 + s + 3


def dopri8_vectors_per_step() -> int:
    """State-sized vectors read + written by one step attempt of the fused 1D1V stepper.

    Stage i < 12 reads its input S_i, y and the K_j (j < i) with a(i+1, j) != 0
    and writes K_i and S_{i+1} (stage 0: S_0 = y); the last stage reads S_12, y
    and the K_j (j < 12) with b_j != 0 or e_j != 0 and writes K_12 and y_new."""
    from .tableau import A, B, E
    total = 3                                                   # stage 0: y; K_0, S_1
    for i in range(1, 12):
        total += 4 + sum(1 for j in A.get(i + 1, {}) if j < i)
    total += 4 + sum(1 for j in range(12) if B[j] != 0 or E[j] != 0)
    return total


def dopri8_combination_fmas_per_entry() -> int:
    """Complex multiply-adds per state entry and step for the stage inputs, y_new and the error."""
    from .tableau import A, B, E
    return sum(len(r) for r in A.values()) + sum(1 for b in B if b) + sum(1 for e in E if e)


def factorize(n: int):
    r = []
    m = n
    while m % 8 == 0:
        r.append(8); m //= 8
    while m % 4 == 0:
        r.append(4); m //= 4
    while m % 2 == 0:
        r.append(2); m //= 2
    p = 3
    while m > 1:
        while m % p == 0:
            r.append(p); m //= p
        p += 2
    return sorted(r, reverse=True)


@dataclass
class Ops:
    instr: float = 0.0   # FP64 instructions (lane ops)
    flops: float = 0.0

    def add(self, fma=0, addmul=0, mult=1.0):
        self.instr += mult * (fma + addmul)
        self.flops += mult * (2 * fma + addmul)


def radix_orders(m: int):
    """Radix orders the plan builder tries for a product-grid length m (csrc/spx_rhs.cu):
    the default factorisation, two 3s merged into a leading 9, and 4 x 4 for 16."""
    f = factorize(m)
    out = [f]
    if f.count(3) >= 2:
        g, skip = [9], 2
        for r in f:
            if r == 3 and skip > 0:
                skip -= 1
                continue
            g.append(r)
        out.append(g)
    if m == 16:
        out.append([4, 4])
    return out


def fft_line_ops(n: int, cut: int | None = None, mode: str = "dit", radices=None) -> Ops:
    """FP64 work of one length-n line through the Stockham engine.

    cut (the 2/3-mask cutoff) prunes the first decimation-in-time stage (masked
    input, mode "dit") or the last decimation-in-frequency stage (masked output,
    mode "dif") when that stage has an odd radix >= 5."""
    o = Ops()
    if n == 1:
        return o
    Ns = 1
    for si, R in enumerate(radices or factorize(n)):
        M = n // R
        tw_tasks = (M - M // Ns) if Ns > 1 else 0
        if R % 2 == 0 or R == 3:
            o.add(fma=2 * (R - 1), addmul=2 * (R - 1), mult=tw_tasks)   # twiddle cmuls
            dft = {2: 4, 3: 12, 4: 16, 8: 56}[R]
            o.add(addmul=dft, mult=M)
        else:
            h = (R - 1) // 2
            prune = cut is not None and si == 0
            qm = [min(h, (cut + j) // M) if prune else h for j in range(M)]
            o.add(fma=4, addmul=4, mult=tw_tasks * h)                   # two twiddles per pair
            if mode == "dit":
                o.add(addmul=4, mult=sum(qm))                           # pair sums / differences
                for q in qm:                                            # all outputs, q <= qmax terms
                    o.add(fma=4 * q, addmul=4, mult=h + 1)
            else:
                o.add(addmul=4, mult=M * h)
                for q in qm:                                            # only outputs kk <= qmax
                    o.add(fma=4 * h, addmul=4, mult=q + 1)
        Ns *= R
    return o


def rhs_ops(shape, tile=None, ntiles=None, product_grid=None, packed=False, radices=None) -> Ops:
    """FP64 work of one right-hand-side evaluation (fused 1D1V or general path).
    product_grid: length of the 1D1V products' grid (the plan's; default Nx),
    transformed with `radices` (the plan's Stockham radices, Plan.product_radices;
    default: the cheapest of the orders the FP64-count rule tries).
    packed (1D1V, exactly Hermitian state): the work the stage kernels execute
    with packed real transforms -- two real lines per complex transform, per tile
    of nt planes ceil((nt + 1) / 2) inverse and ceil(nt / 2) forward transforms,
    and only the k <= 0 half of each output plane evaluated."""
    Nx, Ny, Nz, Nn, Nm, Np, Ns = shape
    o = Ops()
    plane = Nx * Ny * Nz
    if Ny == 1 and Nz == 1 and Nm == 1 and Np == 1:
        cut = Nx // 3
        M = product_grid or Nx
        if radices:
            rad = list(radices)
        elif M == Nx:
            rad = factorize(Nx)
        else:
            rad = min(radix_orders(M), key=lambda r: fft_line_ops(M, cut, "dit", r).instr +
                      fft_line_ops(M, cut, "dif", r).instr)
        fi, ff = fft_line_ops(M, cut, "dit", rad), fft_line_ops(M, cut, "dif", rad)
        ntiles = ntiles or 1
        if packed:
            T = tile or -(-Nn // ntiles)
            nts = [min(T, Nn - t * T) for t in range(ntiles)]
            lines_inv = Ns * sum((nt + 2) // 2 for nt in nts)
            lines_fwd = Ns * sum((nt + 1) // 2 for nt in nts)
            o.add(addmul=2, mult=lines_fwd * M)                      # packed real products
            o.add(fma=6, addmul=6, mult=Ns * Nn * ((Nx + 1) // 2))   # half plane + the packed split
        else:
            lines_inv = Ns * (Nn + ntiles)          # C_{n-1} per plane + one G per tile
            lines_fwd = Ns * Nn
            o.add(fma=2, addmul=2, mult=Ns * Nn * M)             # G * C
            o.add(fma=6, addmul=4, mult=Ns * Nn * Nx)            # streaming, damping, NL add
        o.instr += fi.instr * lines_inv + ff.instr * lines_fwd
        o.flops += fi.flops * lines_inv + ff.flops * lines_fwd
        o.add(fma=4, addmul=2, mult=Ns * Nx)                 # G combination
        o.add(fma=8 * Ns + 6, addmul=24, mult=Nx)            # Maxwell + current
        return o
    def plane_ops(mode):
        fy, fx, fz = (fft_line_ops(N, N // 3, mode) for N in (Ny, Nx, Nz))
        return Ops(instr=fy.instr * Nx * Nz + fx.instr * Ny * Nz + fz.instr * Ny * Nx,
                   flops=fy.flops * Nx * Nz + fx.flops * Ny * Nz + fz.flops * Ny * Nx)
    pi, pf = plane_ops("dit"), plane_ops("dif")
    nplanes = Ns * Nn * Nm * Np
    o.instr += pi.instr * (nplanes + 3 * Ns + 3) + pf.instr * nplanes
    o.flops += pi.flops * (nplanes + 3 * Ns + 3) + pf.flops * nplanes
    o.add(fma=30, addmul=12, mult=nplanes * plane)           # real-space bracket (interior planes)
    o.add(fma=12, addmul=8, mult=nplanes * plane)            # streaming x/y/z, damping, NL add
    o.add(fma=8 * Ns + 6, addmul=24, mult=plane)
    return o


def state_len(shape) -> int:
    Nx, Ny, Nz, Nn, Nm, Np, Ns = shape
    return Ns * Nn * Nm * Np * Nx * Ny * Nz + 6 * Nx * Ny * Nz
