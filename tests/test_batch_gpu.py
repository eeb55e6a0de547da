"""GPU: the batched persistent solver against single-instance solves and the oracle."""
import numpy as np
import pytest

from conftest import rel_err


def _small_insts(seed=0):
    from spectrax_gb300.batch import landau_scan
    insts = landau_scan(n=6, seed=seed)
    # shrink the Hermite axis so the oracle comparison stays quick
    from spectrax_gb300.params import make_problem
    out = []
    rng = np.random.default_rng(seed + 1)
    for it, (Nx, Nn) in zip(insts, [(9, 8), (17, 16), (33, 24), (17, 6), (9, 30), (33, 12)]):
        k = it["k"]
        L = 2 * np.pi / k
        pb = make_problem(Nx, 1, 1, Nn, 1, 1, 2, [-1.0, 1.0], it["nu"], 0.0, [1.0, 1 / 1836.0],
                          [np.sqrt(2)] * 3 + [np.sqrt(2 / 1836.0)] * 3, [0.0] * 6, L, 1.0, 1.0, "divide")
        n = 2 * Nn * Nx + 6 * Nx
        y0 = np.zeros(n, np.complex128)
        c0 = (Nx - 1) // 2
        y0[c0] = 1 / np.sqrt(2) ** 3
        y0[c0 - 1], y0[c0 + 1] = 0.005j, -0.005j
        y0[Nn * Nx + c0] = 1 / np.sqrt(2 / 1836.0) ** 3
        y0[2 * Nn * Nx + c0 - 1] = y0[2 * Nn * Nx + c0 + 1] = 0.01 * L / (4 * np.pi)
        y0[: 2 * Nn * Nx] += 1e-4 * (rng.standard_normal(2 * Nn * Nx) + 1j * rng.standard_normal(2 * Nn * Nx))
        out.append(dict(problem=pb, y0=y0, masses=[1.0, 1836.0], shape=(Nx, 1, 1, Nn, 1, 1, 2), L=L, nu=it["nu"]))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("cluster,tile", [(1, 8), (2, 4), (4, 8), (8, 16), (8, -1), (16, -1)])
def test_batch_matches_serial(cluster, tile):
    import torch
    from spectrax_gb300.batch import BatchSolver, serial_solve
    insts = _small_insts()
    ts = np.linspace(0, 1.0, 5)
    ref_y, ref_st, ref_en, _ = serial_solve(insts, 1.0, dt0=0.01, rtol=1e-9, atol=1e-9, save_ts=ts)
    b = BatchSolver([it["problem"] for it in insts], 1.0, dt0=0.01, rtol=1e-9, atol=1e-9, save_ts=ts,
                    cluster=cluster, tile=tile, masses=[it["masses"] for it in insts])
    yout = b.run(b.pack([it["y0"] for it in insts]))
    torch.cuda.synchronize()
    ys = b.unpack(yout)
    stats, ens = b.results()
    for i in range(len(insts)):
        assert stats[i]["status"] == 1, stats[i]
        assert rel_err(ys[i], ref_y[i]) < 1e-9, (i, rel_err(ys[i], ref_y[i]))
        np.testing.assert_allclose(ens[i][:, 0], ref_en[i][:, 0], rtol=1e-9)
        assert abs(stats[i]["accepted"] - ref_st[i]["accepted"]) <= 1


@pytest.mark.gpu
@pytest.mark.parametrize("saveat", ["interpolate", "land"])
def test_batch_save_modes_match_oracle(saveat):
    # energies at 21 save times (several inside one step when interpolating)
    # against the oracle's states in the same save mode; identical step counts
    from oracle import diag as odiag
    from oracle import dopri8 as od
    from oracle import rhs as orhs
    from oracle import tables as otab
    from spectrax_gb300.batch import BatchSolver
    insts = _small_insts(2)[:3]
    ts = np.linspace(0.0, 0.6, 21)
    # dt0 and tolerances keep every step's error norm far above rounding noise
    # (a noise-level norm would let GPU and oracle propose different steps)
    b = BatchSolver([it["problem"] for it in insts], 0.6, dt0=0.1, rtol=1e-12, atol=1e-12, save_ts=ts,
                    cluster=2, tile=4, masses=[it["masses"] for it in insts], saveat=saveat)
    b.unpack(b.run(b.pack([it["y0"] for it in insts])))
    stats, ens = b.results()
    for i, it in enumerate(insts):
        pb = it["problem"]
        user = dict(Lx=pb.Lx, nu=pb.nu, qs=[-1.0, 1.0], alpha_s=list(pb.alpha_s)[:6], u_s=[0.0] * 6,
                    Omega_cs=[1.0, 1 / 1836.0], mi_me=1836.0)
        p = otab.initialize_simulation_parameters(user, *it["shape"], 5, 0.02)
        ref = od.solve(lambda t, y: orhs.rhs(p, y), 0.0, 0.6, it["y0"], 0.1, ts=ts, adaptive=True,
                       rtol=1e-12, atol=1e-12, saveat=saveat)
        assert stats[i]["accepted"] == ref["accepted"] and stats[i]["rejected"] == ref["rejected"]
        assert stats[i]["saved"] == len(ts)
        Nx, Ny, Nz, Nn, Nm, Np, Ns = it["shape"]
        e_ref = odiag.energies(ref["ys"], Nx, Ny, Nz, Nn, Nm, Np, Ns, p["alpha_s"], p["u_s"], p["Omega_cs"],
                               mi_me=1836.0)
        np.testing.assert_allclose(ens[i][:, 0], e_ref["EM_energy"], rtol=1e-9)
        np.testing.assert_allclose(ens[i][:, 1], e_ref["kinetic_energy"].real, rtol=1e-9)


@pytest.mark.gpu
def test_batch_matches_oracle():
    import torch
    from oracle import dopri8 as od
    from oracle import rhs as orhs
    from oracle import tables as otab
    from spectrax_gb300.batch import BatchSolver
    insts = _small_insts(3)[:2]
    b = BatchSolver([it["problem"] for it in insts], 0.5, dt0=0.02, rtol=1e-10, atol=1e-10,
                    save_ts=np.array([0.25, 0.5]), cluster=2, tile=4)
    ys = b.unpack(b.run(b.pack([it["y0"] for it in insts])))
    stats, _ = b.results()
    for i, it in enumerate(insts):
        pb = it["problem"]
        user = dict(Lx=pb.Lx, nu=pb.nu, qs=[-1.0, 1.0], alpha_s=list(pb.alpha_s)[:6], u_s=[0.0] * 6,
                    Omega_cs=[1.0, 1 / 1836.0])
        p = otab.initialize_simulation_parameters(user, *it["shape"], 5, 0.02)
        ref = od.solve(lambda t, y: orhs.rhs(p, y), 0.0, 0.5, it["y0"], 0.02, ts=np.array([0.25, 0.5]),
                       adaptive=True, rtol=1e-10, atol=1e-10)
        assert rel_err(ys[i], ref["ys"][-1]) < 1e-9
        assert stats[i]["accepted"] == ref["accepted"]


@pytest.mark.gpu
def test_batch_status_and_reuse():
    import torch
    from spectrax_gb300.batch import BatchSolver
    insts = _small_insts(5)[:3]
    b = BatchSolver([it["problem"] for it in insts], 1.0, dt0=0.001, rtol=1e-9, atol=1e-9,
                    max_steps=7, cluster=1, tile=8)
    y0 = b.pack([it["y0"] for it in insts])
    for _ in range(2):                     # the captured graph can be replayed
        b.run(y0)
        stats, _ = b.results()
        assert all(s["status"] == 2 and s["accepted"] == 7 for s in stats)


def _hermitian(y, Nx):
    L = np.array(y, np.complex128).reshape(-1, Nx)
    c0 = Nx // 2
    L[:, c0] = L[:, c0].real
    L[:, :c0] = np.conj(L[:, ::-1][:, :c0])
    return L.ravel()


@pytest.mark.gpu
def test_batch_hermitian_instances():
    # exactly Hermitian initial states (odd Nx) take the packed real-transform tiles
    import torch
    from spectrax_gb300.batch import BatchSolver, serial_solve
    insts = _small_insts(7)
    for it in insts:
        it["y0"] = _hermitian(it["y0"], it["shape"][0])
    ts = np.linspace(0, 1.0, 3)
    ref_y, ref_st, ref_en, _ = serial_solve(insts, 1.0, dt0=0.01, rtol=1e-9, atol=1e-9, save_ts=ts)
    for herm in (True, False):
        b = BatchSolver([it["problem"] for it in insts], 1.0, dt0=0.01, rtol=1e-9, atol=1e-9, save_ts=ts,
                        cluster=2, tile=4, masses=[it["masses"] for it in insts], hermitian=herm)
        ys = b.unpack(b.run(b.pack([it["y0"] for it in insts])))
        stats, ens = b.results()
        for i, it in enumerate(insts):
            assert stats[i]["hermitian"] == herm
            assert rel_err(ys[i], ref_y[i]) < 1e-9, (herm, i)
            np.testing.assert_allclose(ens[i][:, 0], ref_en[i][:, 0], rtol=1e-9)
            L = ys[i].reshape(-1, it["shape"][0])
            if herm:
                assert np.all(L == np.conj(L[:, ::-1]))          # symmetry kept exactly


@pytest.mark.gpu
def test_autotune_refines_the_fastest_candidates():
    # the sweep over (cluster, tile) at a short horizon, then the fastest two again
    # over a longer one; the choice is one of the refined candidates
    from spectrax_gb300.batch import autotune, landau_scan
    insts = landau_scan(12, seed=3)
    best = autotune([it["problem"] for it in insts], [it["y0"] for it in insts], t1_probe=0.05,
                    masses=[it["masses"] for it in insts], clusters=(1, 2), tiles=(4, 8), use_cache=False,
                    refine=2, t1_refine=0.1)
    assert len(best["table"]) == 4 and len(best["refined"]) == 2
    assert (best["cluster"], best["tile"]) in {(r["cluster"], r["tile"]) for r in best["refined"]}
    fastest_two = sorted(best["table"], key=lambda r: r["ms"])[:2]
    assert {(r["cluster"], r["tile"]) for r in fastest_two} == {(r["cluster"], r["tile"]) for r in best["refined"]}
