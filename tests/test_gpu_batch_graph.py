"""Batched form on the GPU: steps launched as a CUDA graph and the autotuner."""

import numpy as np
import pytest

from opensurgsim_gb300 import _lib, mesh

pytestmark = pytest.mark.gpu

DIMS = [(2, 2, 3, 1e4), (4, 3, 2, 1e5), (1, 1, 1, 3e5), (5, 5, 6, 1e6), (3, 6, 2, 2e4)]


def _batch(**kw):
    from opensurgsim_gb300.body import Body

    scenes = [mesh.scene_cube(a, b, c, seed=k, young=float(E)) for k, (a, b, c, E) in enumerate(DIMS)]
    b = Body([s.mesh for s in scenes], rayleigh_mass=0.01, rayleigh_stiffness=0.001, gravity=(0, 0, -9.81),
             cg_tolerance=1e-10, precision=_lib.PRECISION_MIXED, **kw)
    v0 = np.random.default_rng(3).normal(0, 0.01, b.n)
    b.set_state(None, v0)
    return scenes, b


def test_graph_steps_equal_regular_steps_bit_for_bit(gpu_lib):
    _, a = _batch()
    _, g = _batch()
    g.set_tuning(*a.tuning())
    assert a.step(1e-3, 6) == _lib.GBFEM_OK
    assert g.step(1e-3, 2, _lib.STEP_GRAPH) == _lib.GBFEM_OK   # captures the graph
    assert g.step(1e-3, 4, _lib.STEP_GRAPH) == _lib.GBFEM_OK   # relaunches it
    xa, va = a.state()
    xg, vg = g.state()
    assert np.array_equal(xa, xg) and np.array_equal(va, vg)
    sg = g.segment_stats()
    assert np.all(sg["converged"] == 1) and np.all(sg["iterations"] > 0)
    # Per graph step: node pass, element update, assembly, right-hand side, solve, state update,
    # validity check, statistics.
    assert g.stats()["kernel_launches"] == 4 * 8


def test_graph_is_recaptured_when_dt_changes(gpu_lib):
    _, a = _batch()
    _, g = _batch()
    g.set_tuning(*a.tuning())
    for dt in (1e-3, 5e-4, 1e-3):
        assert a.step(dt, 2) == _lib.GBFEM_OK
        assert g.step(dt, 2, _lib.STEP_GRAPH) == _lib.GBFEM_OK
    assert np.array_equal(a.state()[0], g.state()[0])


def test_graph_step_reports_a_nonfinite_state(gpu_lib):
    _, g = _batch()
    x, v = g.state()
    v[7] = np.nan
    g.set_state(None, v)
    assert g.step(1e-3, 3, _lib.STEP_GRAPH) == _lib.GBFEM_NONFINITE
    assert g.step(1e-3, 1, _lib.STEP_GRAPH) == _lib.GBFEM_INACTIVE


def test_autotune_picks_a_candidate_and_pinning_reproduces_it(gpu_lib):
    scenes, t = _batch(autotune=True)
    _, ref = _batch()
    assert t.step(1e-3, 3) == _lib.GBFEM_OK
    assert ref.step(1e-3, 3) == _lib.GBFEM_OK
    e, c, r, g = t.tuning()
    assert e in (32, 64) and c in (2, 3, 4) and r in (1, 2, 3, 4)
    assert g in (_lib.CG_TWO_PHASE, _lib.CG_ONE_PHASE)
    xt, _ = t.state()
    xr, _ = ref.state()
    for k, s in enumerate(scenes):
        n0, n1 = t.node_offsets[k], t.node_offsets[k + 1]
        x0 = s.mesh.nodes.ravel()
        d = xr[3 * n0:3 * n1] - x0
        assert np.linalg.norm(xt[3 * n0:3 * n1] - x0 - d) <= 1e-6 * np.linalg.norm(d)
    # A second body pinned to the tuned choice repeats the tuned run bit for bit.
    _, p = _batch()
    p.set_tuning(e, c, r, g)
    assert p.step(1e-3, 3) == _lib.GBFEM_OK
    assert np.array_equal(p.state()[0], xt)


def test_autotune_with_graph_steps(gpu_lib):
    _, t = _batch(autotune=True)
    assert t.step(1e-3, 4, _lib.STEP_GRAPH) == _lib.GBFEM_OK
    assert t.stats()["steps"] == 4
    assert np.all(t.segment_stats()["converged"] == 1)


def test_set_tuning_rejects_bad_values(gpu_lib):
    _, b = _batch()
    before = b.tuning()
    with pytest.raises(_lib.GbfemError):
        b.set_tuning(48, 2, 6)
    with pytest.raises(_lib.GbfemError):
        b.set_tuning(64, 5, 6)
    with pytest.raises(_lib.GbfemError):
        b.set_tuning(64, 2, 2, _lib.CG_FP64)  # the FP64 schedule on a mixed batch
    with pytest.raises(_lib.GbfemError):
        b.set_tuning(64, 2, 2, 9)
    assert b.tuning() == before  # a rejected call leaves the tuning as it was


def test_timed_graph_steps_report_the_solve_time(gpu_lib):
    _, a = _batch()
    _, g = _batch()
    g.set_tuning(*a.tuning())
    assert a.step(1e-3, 3) == _lib.GBFEM_OK
    assert g.step(1e-3, 3, _lib.STEP_GRAPH | _lib.STEP_TIME_KERNELS) == _lib.GBFEM_OK
    st = g.stats()
    assert st["spmv_timed"] == 3 and st["ms_spmv"] > 0.0
    assert np.array_equal(a.state()[0], g.state()[0])


def test_default_cg_cap_is_per_mesh(gpu_lib):
    """With tolerance 0 no mesh converges, so each stops at its own cap 2 n_mesh + 64 (as each
    representation's own solver would), not at the batch's 2 n + 64."""
    from opensurgsim_gb300.body import Body

    scenes = [mesh.scene_cube(a, b, c, seed=k, young=float(E)) for k, (a, b, c, E) in enumerate(DIMS)]
    b = Body([s.mesh for s in scenes], gravity=(0, 0, -9.81), cg_tolerance=0.0, precision=_lib.PRECISION_MIXED)
    assert b.step(1e-3, 1) == _lib.GBFEM_CG_MAXITER
    st = b.segment_stats()
    it, conv = st["iterations"], st["converged"]
    caps = [2 * 3 * s.mesh.num_nodes + 64 for s in scenes]
    assert not conv.any()
    for k, cap in enumerate(caps):
        assert cap - 2 <= it[k] <= cap, (k, it[k], cap)
    assert max(caps) < 2 * b.n + 64


def test_thousands_of_tiny_meshes_on_one_cta_per_sm(gpu_lib):
    """5,000 one-chunk meshes on a grid of one CTA per SM: each CTA's range holds more meshes than
    the solve's per-phase shared-memory scalar cache (those beyond it read their scalars from
    global memory), and every mesh must still match the oracle."""
    from oracle import oracle as O
    from opensurgsim_gb300.body import Body

    kw = dict(rayleigh_mass=0.01, rayleigh_stiffness=0.001, gravity=(0, 0, -9.81), cg_tolerance=1e-10)
    scenes = [mesh.scene_cube(1 + k % 2, 1 + (k // 2) % 2, 1 + (k // 4) % 2, seed=k, young=1e4 * (1 + k % 97))
              for k in range(5000)]
    b = Body([s.mesh for s in scenes], precision=_lib.PRECISION_MIXED, **kw)
    b.set_tuning(64, 1, 2)
    assert b.step(1e-3, 2) == _lib.GBFEM_OK
    x, _ = b.state()
    assert b.segment_stats()["converged"].all()
    for k in range(0, 5000, 199):
        s = scenes[k]
        o = O.OracleModel(s.mesh, **kw)
        assert o.step(1e-3, 2) == 0
        ox, _ = o.state()
        n0, n1 = b.node_offsets[k], b.node_offsets[k + 1]
        x0 = s.mesh.nodes.ravel()
        u, uo = x[3 * n0:3 * n1] - x0, ox - x0
        assert np.linalg.norm(u - uo) <= 1e-6 * np.linalg.norm(uo), k
