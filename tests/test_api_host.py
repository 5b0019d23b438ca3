"""Host-side logic of the Genesis-style facade (no GPU): options, materials, morph sampling,
derived solver constants, workload generators and the serving admission arithmetic."""

import math

import numpy as np
import pytest

import genesis_gb300 as gs
from genesis_gb300 import morphs
from genesis_gb300.exceptions import GenesisException


def test_sim_and_mpm_options_defaults_and_validation():
    so = gs.options.SimOptions()
    assert so.dt == 1e-2 and so.substeps == 1 and so.substeps_local == 1 and so.gravity == (0.0, 0.0, -9.81)
    mo = gs.options.MPMOptions()
    assert mo.grid_density == 64 and mo.particle_size == pytest.approx(0.01)
    assert gs.options.MPMOptions(grid_density=128).particle_size == pytest.approx(0.005)
    with pytest.raises(GenesisException, match="upper_bound"):
        gs.options.MPMOptions(lower_bound=(0, 0, 1), upper_bound=(1, 1, 0))
    with pytest.raises(GenesisException):
        gs.options.SimOptions(nonsense=1)
    with pytest.raises(GenesisException, match="divisible"):
        gs.options.SimOptions(requires_grad=True, substeps=3, substeps_local=4)
    # MPMOptions inherits dt and gravity from SimOptions (scene.py:157)
    merged = gs.options.MPMOptions().model_copy_from(gs.options.SimOptions(dt=3e-4, gravity=(0, 0, -1)))
    assert merged.dt == 3e-4 and merged.gravity == (0, 0, -1)


def test_material_defaults_match_reference_formulas():
    e = gs.materials.MPM.Elastic()
    assert e.E == 3e5 and e.nu == 0.2 and e.rho == 1000.0
    assert e.mu == pytest.approx(3e5 / (2 * 1.2)) and e.lam == pytest.approx(3e5 * 0.2 / (1.2 * 0.6))
    assert gs.materials.MPM.Liquid().mu == 0.0
    assert gs.materials.MPM.Liquid(viscous=True).mu > 0
    s = gs.materials.MPM.Sand()
    sp = math.sin(math.radians(45.0))
    assert s.alpha == pytest.approx(math.sqrt(2 / 3) * 2 * sp / (3 - sp)) and s._default_Jp == 0.0
    sn = gs.materials.MPM.Snow()
    assert sn.yield_lower == 2.5e-2 and sn.yield_higher == 4.5e-3 and not sn.use_von_mises
    with pytest.raises(GenesisException):
        gs.materials.MPM.Snow(use_von_mises=True)
    m = gs.materials.MPM.Muscle()
    assert m.E == 1e6 and m.model == "neohooken" and m.stiffness == 1e6
    ep = gs.materials.MPM.ElastoPlastic()
    assert ep.use_von_mises and ep.von_mises_yield_stress == 10000.0
    with pytest.raises(GenesisException):
        gs.materials.MPM.Elastic(nu=0.5)
    with pytest.raises(GenesisException):
        gs.materials.MPM.Elastic(sampler="bogus")


def test_material_c_records():
    from genesis_gb300 import _lib

    r = gs.materials.MPM.ElastoPlastic().to_c(3)
    assert r.type == _lib.MAT_ELASTOPLASTIC and r.flags == _lib.MATF_VON_MISES and r.scene == 3
    assert gs.materials.MPM.Elastic(model="neohooken").to_c(0).flags == _lib.MATF_NEOHOOKEAN
    assert gs.materials.MPM.Sand().to_c(0).default_Jp == 0.0


def test_box_regular_sampler_matches_reference_count_and_layout():
    p = morphs.box_to_particles(1 / 128, (0.5, 0.5, 0.4), (0.2, 0.2, 0.2), "regular")
    assert len(p) == 26**3  # n_particles_1D = round(0.2 * 128) = 26 per axis
    assert p.min(0) == pytest.approx(np.array([0.4, 0.4, 0.3]) + 0.5 / 128)
    assert morphs.n_particles_3D(0.01, (0.3, 0.2, 0.1)) == 30 * 20 * 10
    np.random.seed(0)
    r = morphs.box_to_particles(0.01, (0, 0, 0), (0.1, 0.1, 0.1), "random")
    assert len(r) == 1000 and np.all(np.abs(r) <= 0.05)


def test_sphere_and_rotation():
    s = morphs.Sphere(pos=(0.5, 0.5, 0.5), radius=0.1).sample(0.01, "regular")
    assert np.all(np.linalg.norm(s - 0.5, axis=1) <= 0.1 + 1e-12)
    b = morphs.Box(pos=(0, 0, 0), size=(0.2, 0.1, 0.1), euler=(0, 0, 90)).sample(0.01, "regular")
    ext = b.max(0) - b.min(0)
    assert ext[1] == pytest.approx(0.19, abs=1e-9) and ext[0] == pytest.approx(0.09, abs=1e-9)


def test_solver_derived_constants_without_gpu():
    from genesis_gb300.solver import MPMSolver

    class _Sim:
        substeps = 1

    gs.EPS = float(np.finfo(np.float32).eps)
    opts = gs.options.MPMOptions(lower_bound=(0, 0, 0), upper_bound=(1, 1, 1)).model_copy_from(
        gs.options.SimOptions(dt=2e-4))
    s = MPMSolver(None, _Sim(), opts)
    assert tuple(s.grid_res) == (65, 65, 65)
    assert s.dx == 1 / 64 and s.particle_volume == pytest.approx((0.01**3) * 1e3)
    assert s.boundary.lower == pytest.approx(np.float32(3 / 64)) and s.boundary.upper[0] == pytest.approx(61 / 64)
    s.add_material(gs.materials.MPM.Elastic())
    m2 = gs.materials.MPM.Elastic()
    s.add_material(m2)
    s.add_material(gs.materials.MPM.Sand())
    assert m2.idx == 0 and len(s._unique_materials()) == 2
    with pytest.raises(GenesisException, match="1e9"):
        MPMSolver(None, _Sim(), gs.options.MPMOptions(grid_density=2000, lower_bound=(-1, -1, -1),
                                                        upper_bound=(1, 1, 1)).model_copy_from(gs.options.SimOptions()))


def test_workload_generators_are_seeded_and_in_range():
    from genesis_gb300.batched import batched_workload
    from genesis_gb300.serve import grid_blocks, serving_workload

    a = batched_workload(n_scenes=64, seed=1)
    b = batched_workload(n_scenes=64, seed=1)
    assert [s.n_particles for s in a] == [s.n_particles for s in b]
    assert all(2000 <= s.n_particles <= 64000 and 0.1 <= s.extent <= 0.3 for s in a)
    assert len({type(s.material).__name__ for s in a}) == 4
    reqs = serving_workload(n_requests=200, rate_hz=100.0, seed=3)
    arr = np.array([r.arrival for r in reqs])
    assert np.all(np.diff(arr) >= 0) and 0.5 < arr[-1] / 2.0 < 2.0  # ~200 arrivals at 100/s
    assert all(1000 <= r.spec.n_particles <= 500000 and 50 <= r.spec.substeps <= 500 for r in reqs)
    assert {int(r.spec.grid_density) + 1 for r in reqs} == {33, 65, 129}
    assert grid_blocks(129) == 33**3 and grid_blocks(65) == 17**3


def test_vvert_supports_reconstruct_the_vertex_at_rest():
    """particle_entity.py:193-232: the support weights reproduce each visual vertex from the sampled
    particles (affine combination, weights summing to 1), supports ordered by distance."""
    from genesis_gb300.entity import MPMEntity
    from genesis_gb300.solver import MPMSolver

    class _Sim:
        substeps = 1

    class _Scene:
        vis_options = gs.options.VisOptions(n_support_neighbors=8)

    gs.EPS = float(np.finfo(np.float32).eps)
    opts = gs.options.MPMOptions(lower_bound=(0, 0, 0), upper_bound=(1, 1, 1)).model_copy_from(gs.options.SimOptions())
    solver = MPMSolver(_Scene(), _Sim(), opts)
    mat = gs.materials.MPM.Elastic()
    solver.add_material(mat)
    ent = MPMEntity(None, solver, mat, morphs.Box(pos=(0.5, 0.5, 0.5), size=(0.1, 0.1, 0.1)), None, 0.01, 0, 40)
    rng = np.random.default_rng(0)
    verts = 0.5 + rng.uniform(-0.05, 0.05, size=(30, 3))
    ent.set_vverts(verts)
    idx, w = ent._vvert_support_idx - 40, ent._vvert_support_w.astype(np.float64)
    assert idx.shape == (30, 8) and np.allclose(w.sum(1), 1.0, atol=1e-6)
    rec = np.einsum("vj,vjd->vd", w, ent._particles[idx])
    assert np.abs(rec - verts).max() < 1e-5
    d = np.linalg.norm(ent._particles[idx] - verts[:, None], axis=2)
    assert np.all(np.diff(d, axis=1) >= -1e-12)


def test_emitter_geometry_helpers_follow_reference_conventions():
    from genesis_gb300.emitter import axis_angle_R, shell_to_particles, z_up_frame

    eps = float(np.finfo(np.float32).eps)
    for d in ([0, 0, -1], [1, 0, 0], [0.3, -0.4, 0.8], [0, 0, 1]):
        R = z_up_frame(np.array(d, float), eps)
        assert np.allclose(R @ R.T, np.eye(3), atol=1e-12) and np.isclose(np.linalg.det(R), 1.0)
        assert np.allclose(R[:, 2], np.array(d) / np.linalg.norm(d))
    R = z_up_frame(np.array([0.3, -0.4, 0.8]), eps)
    assert abs(R[2, 0]) < 1e-12  # first axis horizontal for a non-vertical direction
    Rz = axis_angle_R([0, 0, 1], 0.5)
    assert np.allclose(Rz, [[np.cos(0.5), -np.sin(0.5), 0], [np.sin(0.5), np.cos(0.5), 0], [0, 0, 1]])
    assert np.allclose(axis_angle_R([0, 0, 1], -0.5), Rz)  # sin from sqrt(1 - cos^2), as the reference
    p = shell_to_particles(0.01, (0, 0, 0), 0.04, 0.1, "regular")
    r = np.linalg.norm(p, axis=1)
    assert len(p) > 0 and r.min() >= 0.04 and r.max() <= 0.1


def test_autotuner_keeps_the_default_shape_within_its_margin():
    from genesis_gb300.autotune import CANDIDATES, DEFAULT, MARGIN, choose

    t = {f"{a}x{b}/{c}": 1.0 for a, b, c in CANDIDATES}
    t["64x2/128"] = 1.0 - MARGIN / 2  # within the margin: noise
    assert choose(t) == DEFAULT
    t["64x2/128"] = 1.0 - 2 * MARGIN  # a clear gain
    assert choose(t) == (64, 2, 128)
    assert choose({"64x2/128": 2.0, "128x1/128": 1.0}, ((64, 2, 128), (128, 1, 128))) == (128, 1, 128)


def _cube_obj(path, half=0.1):
    v = [(x, y, z) for x in (-half, half) for y in (-half, half) for z in (-half, half)]
    # outward-oriented quads (1-based), split into fans by the loader
    quads = [(1, 2, 4, 3), (5, 7, 8, 6), (1, 5, 6, 2), (3, 4, 8, 7), (1, 3, 7, 5), (2, 6, 8, 4)]
    with open(path, "w") as f:
        f.write("# cube\n")
        for p in v:
            f.write("v %f %f %f\n" % p)
        for q in quads:
            f.write("f " + " ".join(f"{i}/{i}/{i}" for i in q) + "\n")


def test_mesh_morph_obj_winding_and_sampling(tmp_path):
    """Mesh morph: OBJ fan triangulation, winding numbers (1 inside, 0 outside a closed mesh), and
    'regular' sampling of a cube mesh equal to the Box morph's lattice (every lattice point lies
    strictly inside), placed by the same pose."""
    import numpy as np

    from genesis_gb300 import morphs

    obj = tmp_path / "cube.obj"
    _cube_obj(obj)
    v, f = morphs.load_obj(obj)
    assert v.shape == (8, 3) and f.shape == (12, 3)
    w = morphs.winding_number(np.array([[0.0, 0.0, 0.0], [0.05, -0.07, 0.02], [0.3, 0.0, 0.0]]), v, f)
    assert abs(w[0] - 1.0) < 1e-9 and abs(w[1] - 1.0) < 1e-9 and abs(w[2]) < 1e-9
    pose = dict(pos=(0.5, 0.4, 0.3), euler=(10.0, 20.0, 30.0))
    mesh = morphs.Mesh(file=str(obj), scale=1.5, **pose)
    box = morphs.Box(size=(0.3, 0.3, 0.3), **pose)
    pm, pb = mesh.sample(0.02, "regular"), box.sample(0.02, "regular")
    assert pm.shape == pb.shape and np.abs(pm - pb).max() < 1e-12
    vv = mesh.visual_vertices()
    assert np.allclose(vv.mean(0), pose["pos"])


def test_mesh_morph_sphere_mesh_counts_close_to_sphere():
    import numpy as np

    from genesis_gb300 import morphs

    # UV sphere of radius 0.1 (outward triangles)
    nu, nv, r = 48, 24, 0.1
    verts = [(0.0, 0.0, r)]
    for i in range(1, nv):
        th = np.pi * i / nv
        for j in range(nu):
            ph = 2 * np.pi * j / nu
            verts.append((r * np.sin(th) * np.cos(ph), r * np.sin(th) * np.sin(ph), r * np.cos(th)))
    verts.append((0.0, 0.0, -r))
    faces = []
    for j in range(nu):
        faces.append((0, 1 + j, 1 + (j + 1) % nu))
    for i in range(nv - 2):
        for j in range(nu):
            a, b = 1 + i * nu + j, 1 + i * nu + (j + 1) % nu
            faces += [(a, a + nu, b), (b, a + nu, b + nu)]
    last = len(verts) - 1
    for j in range(nu):
        a, b = 1 + (nv - 2) * nu + j, 1 + (nv - 2) * nu + (j + 1) % nu
        faces.append((a, last, b))
    mesh = morphs.Mesh(vertices=np.array(verts), faces=np.array(faces))
    n_mesh = len(mesh.sample(0.01, "regular"))
    n_sphere = len(morphs.Sphere(radius=0.1).sample(0.01, "regular"))
    assert abs(n_mesh - n_sphere) <= 0.03 * n_sphere, (n_mesh, n_sphere)


def test_sdf_grid_from_mesh_matches_the_analytic_box():
    """SDFGrid.from_mesh of a box mesh: the reference's normalised frame and [-0.6, 0.6]^3 grid,
    distances to the triangles and winding-number signs equal the exact box SDF there, and
    T_mesh_to_sdf takes the scaled mesh frame to voxel coordinates."""
    import numpy as np

    from genesis_gb300.coupling import SDFGrid

    h = np.array([0.2, 0.1, 0.05])  # half extents; largest extent 0.4 -> normalised half (0.5, 0.25, 0.125)
    v = np.array([(x, y, z) for x in (-h[0], h[0]) for y in (-h[1], h[1]) for z in (-h[2], h[2])]) + 0.3
    quads = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    f = np.array([t for q in quads for t in ((q[0], q[1], q[2]), (q[0], q[2], q[3]))])
    res = 17
    g = SDFGrid.from_mesh(v, f, res=res, scale=2.0)
    hn = h / 0.4
    ax = np.linspace(-0.6, 0.6, res)
    P = np.stack(np.meshgrid(ax, ax, ax, indexing="ij"), -1)
    q = np.abs(P) - hn
    exact = np.linalg.norm(np.maximum(q, 0.0), axis=-1) + np.minimum(q.max(-1), 0.0)
    assert np.abs(g.values - exact).max() < 1e-6
    # a point of the scaled mesh frame (scale 2: normalised coordinates x 2) lands on its voxel
    pn = np.array([0.3, -0.15, 0.6])
    vox = g.T_mesh_to_sdf @ np.append(pn * 2.0, 1.0)
    assert np.allclose(vox[:3], (pn + 0.6) / 1.2 * (res - 1))


def test_custom_force_field_splits_the_field_list_into_grid_op_stages():
    """force_fields.Custom (force_fields.py:424-437): a callable replaces get_acc; it has no device
    record, and the solver's plan runs the built-in fields before it in grid-op stage 1, the Custom
    field, then the built-in fields after it in stage 2."""
    from genesis_gb300.solver import MPMSolver

    ff = gs.force_fields
    with pytest.raises(TypeError):
        ff.Custom(3.0)
    c = ff.Custom(lambda pos, vel, t, i: vel)
    assert c.get_acc is not None and not c.active
    with pytest.raises(TypeError):
        c.to_c()

    class _Lib:
        calls = []

        def mpm_set_force_fields(self, ctx, n, arr):
            self.calls.append(n)
            return 0

    s = MPMSolver.__new__(MPMSolver)
    s._ctx, s._lib = object(), _Lib()
    s._ffs = [ff.Drag(), c, ff.Constant(), ff.Wind(), ff.Custom(lambda p, v, t, i: p)]
    s._upload_force_fields()
    kinds = [p[0] for p in s._ff_plan]
    assert kinds == ["fields", "custom", "fields", "custom", "fields"]
    assert s._ff_plan[0][1:] == (0, 1) and s._ff_plan[2][1:] == (1, 3) and s._ff_plan[4][1:] == (3, 3)
    assert _Lib.calls == [3]
    s._ffs = [ff.Drag()]
    s._upload_force_fields()
    assert s._ff_plan is None


def test_tool_entity_colliders_inputs_and_sdf(tmp_path):
    """Tool entity (tool_entity.py, mesh.py) without a GPU: its SDF is the normalised, scaled mesh's
    (negative at the centre, zero on the faces), it makes one "tool" collider per environment with
    the Tool material's friction and softness and the floor height, inputs set before a step are
    applied by process_input (broadcast over environments), and reset returns it to the morph's
    pose at rest."""
    import numpy as np

    from genesis_gb300.materials import Tool
    from genesis_gb300.tool import ToolEntity, replace_pose

    obj = tmp_path / "cube.obj"
    _cube_obj(obj, half=1.0)
    morph = morphs.Mesh(file=str(obj), scale=0.1, pos=(0.3, 0.1, 0.28), euler=(90.0, 0.0, 0.0))
    mat = Tool(friction=8.0, sdf_res=24)
    with pytest.raises(GenesisException):
        Tool(friction=-1.0)
    t = ToolEntity(scene=None, idx=2, solver=None, material=mat, morph=morph)
    g = t.sdf
    assert g.values.shape == (24, 24, 24) and g.grads is None
    # the cube spans [-0.5, 0.5] after normalisation, scaled by 0.1: its centre maps to the grid centre
    pv = g.T_mesh_to_sdf @ np.array([0.0, 0.0, 0.0, 1.0])
    assert np.allclose(pv[:3], 11.5)
    assert g.values.min() < -0.04 and abs(g.values.min() + 0.5) < 0.05  # distance in normalised units
    t._build(2, floor_height=0.05)
    cols = t._colliders()
    assert [c.env for c in cols] == [0, 1] and all(c.shape == "tool" and c.sdf is g for c in cols)
    assert cols[0].coup_friction == 8.0 and cols[0].coup_softness == 0.01 and cols[0].floor_height == 0.05
    assert np.allclose(cols[1].pos, (0.3, 0.1, 0.28)) and np.allclose(cols[1].quat, morph.quat)
    t.set_velocity(vel=(0.0, 1.0, 0.0))
    t.set_position([[0.3, 0.1, 0.28], [0.3, 0.1, 0.5]])
    assert t._pending()
    t.process_input()
    assert not t._pending()
    assert np.allclose(t._vel, [[0, 1, 0], [0, 1, 0]]) and np.allclose(t._pos[1], (0.3, 0.1, 0.5))
    with pytest.raises(GenesisException):
        t.set_velocity(vel=np.zeros((3, 3)))
        t.process_input()
    t._col0 = 1
    t._sync_pose(np.array([[9.0] * 7, [1, 2, 3, 1, 0, 0, 0], [4, 5, 6, 0, 1, 0, 0]], dtype=np.float64))
    assert np.allclose(t._pos, [[1, 2, 3], [4, 5, 6]]) and np.allclose(t._quat[1], (0, 1, 0, 0))
    t.reset()
    assert np.allclose(t._pos, [(0.3, 0.1, 0.28)] * 2) and not t._vel.any()
    c2 = replace_pose(cols[0], np.array([1.0, 2.0, 3.0, 0.0, 0.0, 0.0, 1.0]))
    assert c2.pos == (1.0, 2.0, 3.0) and c2.quat == (0.0, 0.0, 0.0, 1.0) and c2.coup_friction == 8.0


def test_add_entity_checks_particles_like_the_reference(monkeypatch):
    """particle_entity.py:278-302 (and the Nowhere morph's own validation): an entity without
    particles, or with particles outside the solver boundary (the domain less its safety padding),
    is refused when it is added."""
    monkeypatch.setattr(gs, "_initialized", True)
    monkeypatch.setattr(gs, "EPS", float(np.finfo(np.float32).eps))
    scene = gs.Scene(sim_options=gs.options.SimOptions(dt=2e-4),
                     mpm_options=gs.options.MPMOptions(lower_bound=(0, 0, 0), upper_bound=(1, 1, 1)))
    mat = gs.materials.MPM.Elastic(sampler="regular")
    with pytest.raises(GenesisException, match="must be positive"):
        scene.add_entity(material=mat, morph=gs.morphs.Nowhere(n_particles=0))
    with pytest.raises(GenesisException, match="outside solver boundary"):
        scene.add_entity(material=mat, morph=gs.morphs.Box(pos=(0.98, 0.5, 0.5), size=(0.1, 0.1, 0.1)))
    e = scene.add_entity(material=mat, morph=gs.morphs.Box(pos=(0.5, 0.5, 0.5), size=(0.1, 0.1, 0.1)))
    assert e.n_particles == 1000  # 10 per axis at the default particle size 0.01
