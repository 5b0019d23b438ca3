"""Pin the CPU oracle against golden vectors produced by executing the reference's own MPM code
(tests/golden/make_golden.py): material updates and full substeps (P2G grid, G2P state)."""

import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _mat(O, p, rho=1000.0):
    t, fl, mu, lam, alpha, yl, yh, vm, st = p[:9]
    return O.make_material(int(t), mu, lam, rho, 0.0 if int(t) == 2 else 1.0, alpha, yl, yh, vm, st, int(fl))


def test_materials_match_reference_functions(oracle):
    g = np.load(os.path.join(GOLDEN, "materials.npz"))
    names = sorted({k.split("/")[0] for k in g.files})
    assert len(names) == 9
    for name in names:
        m = _mat(oracle, g[f"{name}/params"])
        moduli = abs(m.lam) + 2 * abs(m.mu) + m.stiffness
        for i in range(len(g[f"{name}/F_tmp"])):
            Fn, jn, P = oracle.material_update(m, g[f"{name}/F_tmp"][i], g[f"{name}/Jp"][i], g[f"{name}/actu"][i],
                                               g[f"{name}/mdir"][i])
            assert np.allclose(Fn, g[f"{name}/F_new"][i], rtol=1e-9, atol=1e-10), (name, i)
            assert abs(jn - g[f"{name}/Jp_new"][i]) <= 1e-9 * max(1, abs(jn)), (name, i)
            assert np.abs(P - g[f"{name}/stress"][i]).max() <= 1e-9 * moduli, (name, i)


@pytest.fixture(scope="module")
def small():
    return np.load(os.path.join(GOLDEN, "substep_small.npz"))


def _oracle_inputs(O, g):
    dt, density, p_size, lx, ly, lz, ux, uy, uz, eps = g["scene"]
    sc = O.make_scene(dt, lower_bound=(lx, ly, lz), upper_bound=(ux, uy, uz), grid_density=density,
                      particle_size=p_size, eps=eps)
    mats = [_mat(O, p, p[9]) for p in g["material_params"]]
    n = len(g["in/pos"])
    st = dict(pos=g["in/pos"], vel=g["in/vel"], C=g["in/C"], F=g["in/F"], Jp=g["in/Jp"], mat=g["in/mat"],
              active=np.ones(n, bool), actu=g["in/actu"], mdir=g["in/mdir"])
    return sc, mats, st


def test_one_substep_grid_and_state(oracle, small):
    sc, mats, st = _oracle_inputs(oracle, small)
    out, grid, _ = oracle.run(sc, mats, st, 1, want_grid=True)
    g1 = small["grid1"]
    assert np.linalg.norm(grid[..., 3] - g1[..., 3]) <= 1e-12 * np.linalg.norm(g1[..., 3])
    assert np.linalg.norm(grid[..., :3] - g1[..., :3]) <= 1e-10 * np.linalg.norm(g1[..., :3])
    for k in ("pos", "vel", "C", "F", "Jp"):
        ref = small["out1/" + k]
        assert np.abs(out[k] - ref).max() <= 1e-9 * max(1.0, np.abs(ref).max()), k


def test_ten_substeps_state(oracle, small):
    sc, mats, st = _oracle_inputs(oracle, small)
    out, _, _ = oracle.run(sc, mats, st, 10)
    for k in ("pos", "vel", "C", "F", "Jp"):
        ref = small["out10/" + k]
        assert np.abs(out[k] - ref).max() <= 1e-8 * max(1.0, np.abs(ref).max()), k


def _golden_fields(g):
    """The facade's force fields built with the fixture's parameters (genesis_gb300.force_fields
    mirrors the constructors of genesis/engine/force_fields.py)."""
    import genesis_gb300.force_fields as ff

    out = []
    for i, name in enumerate(g["fields"]):
        kw = {k.split("/")[1]: g[k] for k in g.files if k.startswith(f"field{i}/")}
        kw = {k: (tuple(v.tolist()) if v.ndim else (int(v) if k == "seed" else float(v))) for k, v in kw.items()}
        f = getattr(ff, str(name))(**kw)
        f.activate()
        out.append(f)
    return out


def test_force_fields_match_reference_code(oracle):
    """The oracle's force fields (Constant, Wind, Point, Drag, Vortex, Turbulence, applied in order
    after gravity in the grid op) against five substeps of the reference's own grid op and field
    code (tests/golden/force_fields.npz)."""
    g = np.load(os.path.join(GOLDEN, "force_fields.npz"))
    sc, mats, st = _oracle_inputs(oracle, g)
    oracle.set_force_fields([f.to_c() for f in _golden_fields(g)])
    try:
        out, grid, _ = oracle.run(sc, mats, st, 1, want_grid=True)
        for k in ("pos", "vel", "C", "F", "Jp"):
            ref = g["out1/" + k]
            assert np.abs(out[k] - ref).max() <= 1e-9 * max(1.0, np.abs(ref).max()), k
        out5, _, _ = oracle.run(sc, mats, st, 5)
    finally:
        oracle.set_force_fields([])
    plain, _, _ = oracle.run(sc, mats, st, 5)
    assert np.abs(plain["vel"] - g["out5/vel"]).max() > 1e-3  # the fields act on this scene
    for k in ("pos", "vel", "C", "F", "Jp"):
        ref = g["out5/" + k]
        assert np.abs(out5[k] - ref).max() <= 1e-8 * max(1.0, np.abs(ref).max()), k


def _golden_colliders(O, g):
    """The facade's colliders for the reference geoms of tests/golden/rigid_coupling.npz (sphere,
    tilted plane, rotated box given by its SDF grid), the box grid registered with the oracle."""
    from genesis_gb300.coupling import Collider, SDFGrid

    out = []
    for i, t in enumerate(g["geom_types"]):
        pos, quat, data = g[f"geom{i}/pos"], g[f"geom{i}/quat"], g[f"geom{i}/data"]
        fr, so, re = g[f"geom{i}/coup"]
        kw = dict(pos=tuple(pos), quat=tuple(quat), lin_vel=tuple(g[f"geom{i}/lin_vel"]),
                  ang_vel=tuple(g[f"geom{i}/ang_vel"]), com=tuple(pos), coup_friction=fr, coup_softness=so,
                  coup_restitution=re)
        sid = -1
        if t == "sphere":
            c = Collider("sphere", radius=float(data[0]), **kw)
        elif t == "plane":
            c = Collider("plane", normal=tuple(data), **kw)
        else:
            grid = SDFGrid(values=g["box_sdf/values"], T_mesh_to_sdf=g["box_sdf/T"], grads=g["box_sdf/grads"],
                           cell_size=float(g["box_sdf/cell_size"]), sdf_max=float(g["box_sdf/sdf_max"]))
            c = Collider("sdf", sdf=grid, **kw)
            sid = O.add_sdf_grid(grid.values, grid.grads, grid.T_mesh_to_sdf, grid.cell_size, grid.sdf_max)
        out.append((c, sid))
    return out


def test_rigid_coupling_matches_reference_code(oracle):
    """The oracle's rigid coupling (SDF of a sphere, a plane and a voxel-SDF box, influence,
    relative-velocity projection with friction and restitution, reaction on the link) against three
    substeps of the reference's own grid op with its rigid-collision, SDF and geometry code
    (tests/golden/rigid_coupling.npz).  The reference accumulates the reaction into the link's
    cfrc_coupling with the opposite sign of the force the oracle reports."""
    g = np.load(os.path.join(GOLDEN, "rigid_coupling.npz"))
    sc, mats, st = _oracle_inputs(oracle, g)
    oracle.clear_sdf_grids()
    cols = _golden_colliders(oracle, g)
    oracle.set_colliders([c.to_c(sid) for c, sid in cols])
    try:
        out, _, _ = oracle.run(sc, mats, st, 3)
        forces = oracle.collider_forces(len(cols))
    finally:
        oracle.set_colliders([])
        oracle.clear_sdf_grids()
    plain, _, _ = oracle.run(sc, mats, st, 3)
    assert np.abs(plain["vel"] - g["out3/vel"]).max() > 1e-3  # the geoms act on this scene
    # both sides run in float64; the remaining differences come from the order of operations
    # (quaternion rotations, normalisations), amplified in C by 4 / dx
    for k in ("pos", "vel", "C", "F", "Jp"):
        ref = g["out3/" + k]
        assert np.abs(out[k] - ref).max() <= 1e-7 * max(1.0, np.abs(ref).max()), k
    assert np.all(np.abs(g["link_force"]).max(1) > 0)
    assert np.abs(forces[:, :3] + g["link_force"]).max() <= 1e-6 * np.abs(g["link_force"]).max()
    assert np.abs(forces[:, 3:] + g["link_torque"]).max() <= 1e-6 * np.abs(g["link_torque"]).max()
