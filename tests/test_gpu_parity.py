"""Parity of the GB300 path with the CPU oracle, through the C ABI.

Integer results (intervals of every mesh id, leaf cells, storage indices,
tags) must be identical; FP64 fields must be bit-identical too, since every
operation is rounded individually in the reference's order (the stated
tolerance of the path is 1e-13 relative; these tests use 0).
"""
import os

import numpy as np
import pytest

from advection_cases import ball_3d, centers, demo_time_loop, disc, readme_square, shapes_2d
from gpu_util import compare_cells, compare_fields, compare_meshes
from oracle.pyoracle import OracleSim

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def sg():
    from samurai_gb300 import build

    build.build()
    import samurai_gb300

    return samurai_gb300


def pair(sg, dim, minl, maxl, pred=1):
    g = sg.AdvectionSim(dim, minl, maxl, 1, pred)
    o = OracleSim(dim, minl, maxl, 1, pred)
    return g, o


def init_both(g, o, f):
    lv, co, _ = o.cells()
    vals = f(lv, co)
    o.set_cell_values(vals)
    g.set_cell_values(vals)


@pytest.mark.parametrize("dim,minl,maxl", [(2, 2, 6), (2, 4, 9), (3, 2, 5)])
def test_uniform_mesh_ids(sg, dim, minl, maxl):
    g, o = pair(sg, dim, minl, maxl)
    compare_meshes(g, o, maxl, "uniform")
    compare_cells(g, o, "uniform")
    assert g.nb_ref() == o.nb_ref()


def test_ghost_update_uniform(sg):
    g, o = pair(sg, 2, 2, 6)
    init_both(g, o, readme_square)
    o.update_ghost()
    g.update_ghost()
    compare_fields(g, o, "ghosts")


@pytest.mark.parametrize("pred", [0, 1])
def test_golden_replay(sg, pred):
    """demos/FiniteVolume/advection_2d.cpp with --Tf 0.01 on the GPU: same
    meshes as the reference's golden files, fields bit-identical to the
    oracle at every step."""
    g, o = pair(sg, 2, 4, 10, pred)
    init_both(g, o, disc)
    o.adapt(2e-4, 1.0)
    g.adapt(2e-4, 1.0)
    compare_cells(g, o, "init")
    compare_fields(g, o, "init", cells_only=True)
    gold = np.load(os.path.join(GOLD, "pred_%d_init.npz" % pred))
    assert np.array_equal(g.cell_values(), gold["u"])
    dt = 0.5 * (1.0 / (1 << 10))
    t, Tf, nt = 0.0, 0.01, 0
    while t != Tf:
        o.adapt(2e-4, 1.0)
        g.adapt(2e-4, 1.0)
        t += dt
        if t > Tf:
            dt += Tf - t
            t = Tf
        o.update_ghost()
        g.update_ghost()
        compare_fields(g, o, "step %d ghosts" % nt)
        o.upwind([1.0, 1.0], dt, 0)
        g.upwind([1.0, 1.0], dt, 0)
        nt += 1
        compare_cells(g, o, "step %d" % nt)
        compare_fields(g, o, "step %d" % nt, cells_only=True)
    compare_meshes(g, o, 10, "final")
    gold = np.load(os.path.join(GOLD, "pred_%d.npz" % pred))
    lv, co, _ = g.cells()
    assert np.array_equal(lv, gold["level"]) and np.array_equal(co[:, 0], gold["i"]) and np.array_equal(co[:, 1], gold["j"])
    np.testing.assert_allclose(g.cell_values(), gold["u"], rtol=1e-14, atol=1e-7)


@pytest.mark.parametrize("scheme", [0, 1])
def test_readme_demo(sg, scheme):
    """README demo (README.md:88-155): min 2, max 8, square of side 0.2, eps
    1e-4, regularity 2, dt = 0.5 dx; all 50 iterations, both upwind forms
    (the upwind operator and the README's lambda)."""
    g, o = pair(sg, 2, 2, 8)
    init_both(g, o, readme_square)
    dt = 0.5 / (1 << 8)
    for it in range(50):
        o.adapt(1e-4, 2.0)
        g.adapt(1e-4, 2.0)
        compare_cells(g, o, "it %d adapt" % it)
        o.update_ghost()
        g.update_ghost()
        o.upwind([1.0, 1.0], dt, scheme)
        g.upwind([1.0, 1.0], dt, scheme)
        compare_fields(g, o, "it %d" % it, cells_only=True)
    compare_meshes(g, o, 8, "readme")


def test_shapes_2d_small(sg):
    """Seeded squares + Gaussians, a = (1, 0.5), min 3, max 8, eps 1e-4, reg 2."""
    g, o = pair(sg, 2, 3, 8)
    init_both(g, o, shapes_2d(7, 6, 6))
    dt = 0.5 / (1 << 8)
    for it in range(6):
        o.adapt(1e-4, 2.0)
        g.adapt(1e-4, 2.0)
        compare_cells(g, o, "shapes it %d" % it)
        o.update_ghost()
        g.update_ghost()
        compare_fields(g, o, "shapes ghosts %d" % it)
        o.upwind([1.0, 0.5], dt, 0)
        g.upwind([1.0, 0.5], dt, 0)
        compare_fields(g, o, "shapes it %d" % it, cells_only=True)
    compare_meshes(g, o, 8, "shapes")


def test_details_and_tags(sg):
    """Detail and tag fields of a converged Harten pass."""
    g, o = pair(sg, 2, 3, 8)
    init_both(g, o, shapes_2d(3, 4, 4))
    o.adapt(1e-4, 2.0)
    g.adapt(1e-4, 2.0)
    # one more pass on the adapted mesh: usually the fixed point
    for ite in range(5):
        ro = o.harten(ite, 1e-4, 2.0)
        rg = g.harten(ite, 1e-4, 2.0)
        assert ro == rg
        if ro:
            do, dg = o.detail(), g.detail()
            assert np.array_equal(do, dg)
            assert np.array_equal(o.tag(), g.tag())
            break
    compare_cells(g, o, "after harten")


def test_3d_small(sg):
    """3D: ball + Gaussians, a = (1,1,1), min 2, max 5, eps 1e-3, reg 1."""
    g, o = pair(sg, 3, 2, 5)
    init_both(g, o, ball_3d(5, 3))
    dt = 0.3 / (1 << 5)
    for it in range(4):
        o.adapt(1e-3, 1.0)
        g.adapt(1e-3, 1.0)
        compare_cells(g, o, "3d it %d" % it)
        o.update_ghost()
        g.update_ghost()
        compare_fields(g, o, "3d ghosts %d" % it)
        o.upwind([1.0, 1.0, 1.0], dt, 0)
        g.upwind([1.0, 1.0, 1.0], dt, 0)
        compare_fields(g, o, "3d it %d" % it, cells_only=True)
    compare_meshes(g, o, 5, "3d")


@pytest.mark.parametrize("dim,minl,maxl,a", [(2, 2, 7, (1.0, 0.7)), (2, 3, 8, (-0.6, 1.0)), (2, 2, 6, (0.0, -1.0)), (3, 2, 5, (0.8, -0.5, 1.0))])
def test_convection_flux_form(sg, dim, minl, maxl, a):
    """make_convection_upwind (flux form, level-jump interfaces) against the
    oracle: meshes and leaf values bit-identical over several adapted steps."""
    g, o = pair(sg, dim, minl, maxl)
    f = shapes_2d(17, 4, 4) if dim == 2 else ball_3d(9)
    init_both(g, o, f)
    dt = 0.4 / (1 << maxl)
    for step in range(4):
        o.adapt(1e-3, 1.0)
        g.adapt(1e-3, 1.0)
        o.update_ghost()
        g.update_ghost()
        o.upwind(a, dt, 2)
        g.upwind(a, dt, sg.CONVECTION)
        compare_cells(g, o, "convection step %d" % step)
        compare_fields(g, o, "convection step %d" % step, cells_only=True)


@pytest.mark.parametrize("dim,minl,maxl,bc", [(2, 2, 7, 0.25), (3, 2, 5, -0.5)])
def test_nonzero_dirichlet(sg, dim, minl, maxl, bc):
    """Dirichlet<1> with a non-zero value: outer ghosts 2v - u, their
    projections and predictions, through adapted steps of both schemes."""
    g = sg.AdvectionSim(dim, minl, maxl, 1, 1, 1, bc)
    o = OracleSim(dim, minl, maxl, 1, 1, 1, bc)
    init_both(g, o, shapes_2d(5, 3, 3) if dim == 2 else ball_3d(4))
    a = (0.75, -1.0) if dim == 2 else (0.5, -0.75, 1.0)
    dt = 0.4 / (1 << maxl)
    for step in range(3):
        for s in (g, o):
            s.adapt(1e-3, 1.0)
            s.update_ghost()
        compare_fields(g, o, "ghosts, step %d" % step)
        scheme = 2 if step == 1 else 0
        o.upwind(a, dt, scheme)
        g.upwind(a, dt, scheme)
        compare_meshes(g, o, maxl, "step %d" % step)
        compare_fields(g, o, "step %d" % step, cells_only=True)


def test_single_level_mesh(sg):
    """min_level == max_level: the adaptation has no pass, the mesh stays
    uniform, and the ghost update and upwind still match."""
    g, o = pair(sg, 2, 5, 5)
    init_both(g, o, readme_square)
    for _ in range(2):
        assert g.adapt(1e-4, 2.0) == 0
        o.adapt(1e-4, 2.0)
        g.update_ghost()
        o.update_ghost()
        g.upwind((1.0, 0.5), 0.5 / 32)
        o.upwind((1.0, 0.5), 0.5 / 32)
    compare_meshes(g, o, 5, "single level")
    compare_fields(g, o, "single level", cells_only=True)


def test_zero_field_coarsens_to_min_level(sg):
    """u = 0: every detail vanishes, the mesh coarsens to min_level."""
    g, o = pair(sg, 2, 3, 8)
    init_both(g, o, lambda lv, co: np.zeros(len(lv)))
    g.adapt(1e-4, 2.0)
    o.adapt(1e-4, 2.0)
    lv, _, _ = g.cells()
    assert np.all(lv == 3)
    compare_meshes(g, o, 8, "zero field")


@pytest.mark.parametrize("dim,minl,maxl,amp", [(2, 2, 8, 1.0), (2, 3, 7, 1e-3), (3, 2, 5, 5.0)])
def test_relative_detail(sg, dim, minl, maxl, amp):
    """mra_config().relative_detail(true): details divided by max |u| over the
    leaf cells before the criteria (mr/rel_detail.hpp), bit for bit."""
    g, o = pair(sg, dim, minl, maxl)
    f = shapes_2d(8, 3, 3) if dim == 2 else ball_3d(6)
    init_both(g, o, lambda lv, co: amp * f(lv, co))
    a = (1.0, -0.5) if dim == 2 else (0.5, 1.0, -0.75)
    dt = 0.4 / (1 << maxl)
    for step in range(3):
        assert g.adapt(1e-3, 1.0, relative_detail=True) == o.adapt(1e-3, 1.0, relative_detail=True)
        compare_meshes(g, o, maxl, "relative detail, step %d" % step)
        for s in (g, o):
            s.update_ghost()
        o.upwind(a, dt)
        g.upwind(a, dt)
        compare_fields(g, o, "relative detail, step %d" % step, cells_only=True)


@pytest.mark.parametrize("dim,minl,maxl", [(2, 2, 7), (3, 2, 5)])
def test_several_fields(sg, dim, minl, maxl):
    """make_MRAdapt(u, v)(mra_config, w): the details of u and v together
    decide the mesh (any component large refines, all small coarsens), u, v
    and the carried field w move to every new mesh; against the oracle,
    meshes and the three fields bit for bit, with a few upwind steps of u."""
    mesh = sg.MRMesh(dim, minl, maxl, 1, 1)
    u, v, w, unp1 = (sg.make_scalar_field(n, mesh) for n in ("u", "v", "w", "unp1"))
    for f, bc in ((u, 0.0), (v, 0.5), (w, -1.0)):
        sg.make_bc(sg.Dirichlet(1), f, bc)
    o = OracleSim(dim, minl, maxl, 1, 1, 1, 0.0)
    kv, kw = o.add_field(0.5), o.add_field(-1.0)
    lv, co, _ = o.cells()
    fu = shapes_2d(3, 2, 2) if dim == 2 else ball_3d(2)
    fv = (lambda l, c: shapes_2d(4, 1, 3)(l, c) * 0.5) if dim == 2 else (lambda l, c: 0.5 * ball_3d(7)(l, c))
    fw = lambda l, c: np.cos(3.0 * centers(l, c)[:, 0])
    for f, k, fun in ((u, 0, fu), (v, kv, fv), (w, kw, fw)):
        vals = fun(lv, co)
        f.set_cells(vals)
        o.set_cell_values_k(k, vals)
    adapt = sg.make_MRAdapt(u, v)
    cfg = sg.mra_config().epsilon(1e-3).regularity(1.0)
    a = (1.0, 0.5) if dim == 2 else (1.0, 0.5, -0.25)
    dt = 0.4 / (1 << maxl)
    for step in range(3):
        assert adapt(cfg, w) == o.adapt_fields(1e-3, 1.0, 2, 1)
        lg, cg, ig = mesh.cells()
        lo_, co_, io_ = o.cells()
        assert np.array_equal(lg, lo_) and np.array_equal(cg, co_) and np.array_equal(ig, io_), "step %d: cells" % step
        for f, k in ((u, 0), (v, kv), (w, kw)):
            got, ref = f.cell_values(), o.cell_values_k(k)
            assert np.array_equal(got, ref), "step %d: field %d differs" % (step, k)
        sg.update_ghost_mr(u, v, w)
        for k in (0, kv, kw):
            o.update_ghost_k(k)
        unp1.assign_upwind(u, a, dt)
        sg.swap(u, unp1)
        o.upwind(a, dt)


@pytest.mark.parametrize("dim,minl,maxl,rel", [(2, 2, 7, False), (2, 3, 8, True), (3, 2, 5, False)])
def test_vector_field(sg, dim, minl, maxl, rel):
    """make_vector_field<double, 3>: make_MRAdapt(v) tests the three detail
    components together (mr/criteria.hpp:45-107; per-component maxima with
    relative details), make_bc gives each component its value, ghosts and
    upwind act component by component, and v.array() keeps samurai's layout
    (the values of a cell side by side).  Against the oracle's several-field
    restatement, bit for bit, with upwind steps."""
    mesh = sg.MRMesh(dim, minl, maxl, 1, 1)
    v = sg.make_vector_field("v", mesh, 3)
    vnp1 = sg.make_vector_field("vnp1", mesh, 3)
    bcs = (0.0, 0.25, -0.5)
    sg.make_bc(sg.Dirichlet(1), v, *bcs)
    sg.make_bc(sg.Dirichlet(1), vnp1, *bcs)
    o = OracleSim(dim, minl, maxl, 1, 1, 1, bcs[0])
    ks = [0, o.add_field(bcs[1]), o.add_field(bcs[2])]
    lv, co, _ = o.cells()
    f0 = shapes_2d(5, 2, 2) if dim == 2 else ball_3d(3)
    f1 = (lambda l, c: 0.5 * shapes_2d(6, 2, 1)(l, c)) if dim == 2 else (lambda l, c: 0.5 * ball_3d(8)(l, c))
    f2 = lambda l, c: 0.1 * np.sin(4.0 * centers(l, c)[:, 1])
    vals = np.stack([f(lv, co) for f in (f0, f1, f2)], axis=1)
    v.set_cells(vals)
    for c, k in enumerate(ks):
        o.set_cell_values_k(k, vals[:, c])
    adapt = sg.make_MRAdapt(v)
    cfg = sg.mra_config().epsilon(1e-3).regularity(1.0).relative_detail(rel)
    a = (1.0, 0.5) if dim == 2 else (1.0, 0.5, -0.25)
    dt = 0.4 / (1 << maxl)
    for step in range(3):
        assert adapt(cfg) == o.adapt_fields(1e-3, 1.0, 3, 0, relative_detail=rel)
        lg, cg, ig = mesh.cells()
        lo_, co_, io_ = o.cells()
        assert np.array_equal(lg, lo_) and np.array_equal(cg, co_) and np.array_equal(ig, io_), "step %d: cells" % step
        got = v.cell_values()
        assert got.shape == (len(lg), 3)
        for c, k in enumerate(ks):
            assert np.array_equal(got[:, c], o.cell_values_k(k)), "step %d: component %d" % (step, c)
        sg.update_ghost_mr(v)
        for k in ks:
            o.update_ghost_k(k)
        full = v.array()
        cells = ig
        for c, k in enumerate(ks):
            ref = o.field_k(k)
            # the reference array holds leaves and ghosts: compare every entry the oracle defines
            m = ~np.isnan(ref)
            assert np.array_equal(full[m, c], ref[m]), "step %d: ghosts of component %d" % (step, c)
        assert np.array_equal(full.reshape(-1)[cells * 3 + 1], got[:, 1])
        vnp1.assign_upwind(v, a, dt)
        sg.swap(v, vnp1)
        for k in ks:
            o.upwind_k(k, a, dt)
    got = v.cell_values()
    for c, k in enumerate(ks):
        assert np.array_equal(got[:, c], o.cell_values_k(k)), "final component %d" % c


@pytest.mark.parametrize("dim,minl,maxl", [(2, 3, 8), (3, 2, 5)])
def test_for_each_interval_and_cell_access(sg, dim, minl, maxl):
    """for_each_interval(mesh, f(level, i, index)) gives the leaf intervals of
    the oracle in samurai's order with their storage offsets, and u(level, i,
    j[, k]) reads the value of a reference cell (a ghost included)."""
    g, o = pair(sg, dim, minl, maxl)
    f = shapes_2d(4, 3, 3) if dim == 2 else ball_3d(4)
    init_both(g, o, f)
    g.adapt(1e-3, 1.0)
    o.adapt(1e-3, 1.0)
    got = []
    sg.for_each_interval(g.mesh, lambda level, i, index: got.append((level, i.start, i.end) + index + (i.index,)))
    ref = []
    for l in range(minl, maxl + 1):
        ref.extend((l,) + tuple(int(v) for v in r) for r in g.mesh.intervals("cells", l, with_index=True))
    assert got == ref
    want = []
    for l in range(minl, maxl + 1):
        want.extend((l,) + tuple(int(v) for v in r) for r in o.intervals("cells", l))
    assert [t[:dim + 2] for t in got] == want
    g.update_ghost()
    field = g.field()
    lv, co, ix = g.cells()
    for k in range(0, len(lv), max(1, len(lv) // 200)):
        assert g.u(int(lv[k]), *[int(c) for c in co[k]]) == field[ix[k]]
    # a ghost: the left neighbour of the first leaf of the finest level
    iv = g.mesh.intervals("reference", maxl, with_index=True)[0]
    e = g.mesh.find(maxl, int(iv[0]), *[int(v) for v in iv[2:dim + 1]])
    assert e == int(iv[dim + 1]) + int(iv[0])
    assert g.u(maxl, int(iv[0]), *[int(v) for v in iv[2:dim + 1]]) == field[e]
    with pytest.raises(IndexError):
        g.u(maxl, -30, *([0] * (dim - 1)))


def test_field_fill_and_factories(sg):
    """u.fill and make_scalar_field with a value or a function of the centre"""
    mesh = sg.MRMesh(2, 2, 6, 1, 1)
    u = sg.make_scalar_field("u", mesh, 1.25)
    assert np.all(u.array() == 1.25)
    v = sg.make_scalar_field("v", mesh, lambda c: c[:, 0] + 2.0 * c[:, 1])
    lv, co, _ = mesh.cells()
    c = centers(lv, co)
    assert np.array_equal(v.cell_values(), c[:, 0] + 2.0 * c[:, 1])
    v.fill(-3.0)
    assert np.all(v.array() == -3.0)


def test_mesh_destroyed_before_its_fields(sg):
    """sg_mesh_destroy of a mesh that still has fields (a reference cycle
    collected in any order, a C caller) releases it with the last field"""
    import ctypes

    L = sg.lib()
    m, f, v = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    assert L.sg_mesh_create(2, 2, 6, 1, 1, 1, ctypes.byref(m)) == 0
    assert L.sg_field_create(m, b"u", ctypes.byref(f)) == 0
    assert L.sg_vector_field_create(m, b"v", 2, ctypes.byref(v)) == 0
    assert L.sg_field_fill(f, 2.0) == 0
    assert L.sg_mesh_set_cells(m, -1, None, None) == 1
    assert L.sg_mesh_destroy(m) == 0
    assert L.sg_vector_field_destroy(v) == 0
    assert L.sg_field_destroy(f) == 0
    # the library and the device stay usable
    g = sg.AdvectionSim(2, 2, 6, 1, 1)
    o = OracleSim(2, 2, 6, 1, 1)
    init_both(g, o, disc)
    assert g.adapt(1e-3, 1.0) == o.adapt(1e-3, 1.0)
    compare_cells(g, o, "after the out-of-order destruction")


@pytest.mark.parametrize("dim", [2, 3])
def test_refine_boundary(sg, dim):
    """--refine-boundary (keep_boundary_refined, mr/adapt.hpp:245-274): the
    boundary leaves of max_level are tagged keep in every pass; meshes, tags
    and values bit-identical to the oracle through the adaptation and steps"""
    minl, maxl = (3, 8) if dim == 2 else (2, 5)
    g, o = pair(sg, dim, minl, maxl)
    g.mesh.set_refine_boundary(True)
    o.set_refine_boundary(True)
    init_both(g, o, shapes_2d(17, 6, 6) if dim == 2 else ball_3d(9))
    a = [1.0, -0.5] if dim == 2 else [1.0, -0.5, 0.25]
    dt = 0.25 / (1 << maxl)
    assert g.adapt(1e-3, 1.0) == o.adapt(1e-3, 1.0)
    for it in range(4):
        compare_cells(g, o, "it %d" % it)
        compare_fields(g, o, "it %d" % it, cells_only=True)
        g.update_ghost()
        o.update_ghost()
        g.upwind(a, dt)
        o.upwind(a, dt)
        assert g.adapt(1e-3, 1.0) == o.adapt(1e-3, 1.0)
    compare_meshes(g, o, maxl, "refine boundary")
    compare_cells(g, o, "final")
    compare_fields(g, o, "final", cells_only=True)
    for ite in range(maxl - minl):
        ro, rg = o.harten(ite, 1e-3, 1.0), g.harten(ite, 1e-3, 1.0)
        assert ro == rg
        if ro:
            assert np.array_equal(o.tag(), g.tag()), "tags of the converged pass"
            break


def test_mesh_beyond_device_memory_is_refused(sg):
    """3D max_level 12: the dense level slabs of the mesh and of one field need
    about 2.3 TB, more than the device holds: SG_ERR_CAPACITY (status 3) with
    the sizes, before any allocation"""
    with pytest.raises(sg.SamuraiGpuError, match=r"status 3\).*GB of device memory"):
        sg.MRMesh(3, 3, 12)
    # the device is still usable
    m = sg.MRMesh(2, 2, 5)
    assert m.nb_cells("cells") == 32 * 32


@pytest.mark.parametrize("dim,minl,maxl", [(2, 2, 9), (3, 2, 6)])
def test_adaptation_graph_matches_pass_by_pass(sg, dim, minl, maxl):
    """the adaptation as one graph with device-side conditions and pass by
    pass with host tests (the default) give identical meshes, values and pass
    counts, from a uniform start (many passes, graduation loops) and along steps"""
    a_graph = sg.AdvectionSim(dim, minl, maxl)
    a_pass = sg.AdvectionSim(dim, minl, maxl)
    a_graph.mesh.set_adapt_graph(True)
    a_pass.mesh.set_adapt_graph(False)
    assert a_graph.mesh.launch_shape()["graphed_adapt"] and not a_pass.mesh.launch_shape()["graphed_adapt"]
    lv, co, _ = a_graph.cells()
    f = shapes_2d(23, 8, 8) if dim == 2 else ball_3d(11)
    for s in (a_graph, a_pass):
        s.set_cell_values(f(lv, co))
    vel = [1.0, -0.75] if dim == 2 else [1.0, -0.75, 0.5]
    dt = 0.3 / (1 << maxl)
    for it in range(6):
        assert a_graph.adapt(1e-4, 2.0) == a_pass.adapt(1e-4, 2.0), "it %d: Harten passes" % it
        lg, cg, ig = a_graph.cells()
        lp, cp, ip = a_pass.cells()
        assert np.array_equal(lg, lp) and np.array_equal(cg, cp) and np.array_equal(ig, ip), "it %d: cells" % it
        assert np.array_equal(a_graph.field(), a_pass.field()), "it %d: field with ghosts" % it
        for s in (a_graph, a_pass):
            s.update_ghost()
            s.upwind(vel, dt)


@pytest.mark.parametrize("dim,scheme,graphed", [(2, 0, True), (2, 1, True), (2, 2, True), (3, 0, True), (2, 0, False), (3, 0, False)])
def test_step_graph_matches_separate_calls(sg, dim, scheme, graphed):
    """sg_step (the whole time step as one graph on the graphed adaptation
    path, the per-pass graphs otherwise) gives what adapt, update_ghost_mr,
    upwind and swap give as separate pass-by-pass calls, bit for bit,
    including the first step from the uniform mesh, whose last Harten pass
    still changes the mesh"""
    minl, maxl = (2, 8) if dim == 2 else (2, 5)
    s_one, s_sep = sg.AdvectionSim(dim, minl, maxl), sg.AdvectionSim(dim, minl, maxl)
    s_one.mesh.set_adapt_graph(graphed)
    s_sep.mesh.set_adapt_graph(False)
    lv, co, _ = s_one.cells()
    f = shapes_2d(29, 6, 6) if dim == 2 else ball_3d(13)
    for s in (s_one, s_sep):
        s.set_cell_values(f(lv, co))
    vel = [1.0, -0.5] if dim == 2 else [1.0, -0.5, 0.75]
    dt = 0.3 / (1 << maxl)
    for it in range(8):
        eps = 1e-4 if it % 3 else 5e-3
        p1 = s_one.step(eps, 2.0, vel, dt, scheme)
        p2 = s_sep.adapt(eps, 2.0)
        s_sep.update_ghost()
        s_sep.upwind(vel, dt, scheme)
        assert p1 == p2, "it %d: Harten passes" % it
        lg, cg, ig = s_one.cells()
        lp, cp, ip = s_sep.cells()
        assert np.array_equal(lg, lp) and np.array_equal(cg, cp) and np.array_equal(ig, ip), "it %d: cells" % it
        assert np.array_equal(s_one.cell_values(), s_sep.cell_values()), "it %d: values" % it
