"""The CUDA substep against golden vectors from the reference's own MPM code (tests/golden/).

Float32 kernels vs float64 reference execution, same inputs: grid mass/momentum after the
first P2G within 1e-5 relative (L2); particle state after 1 and 10 substeps within float32
tolerances stated below."""

import os

import numpy as np
import pytest
import torch

from capi_helpers import Ctx, material_record, scene_record

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def ctx():
    import __graft_entry__ as g

    g.build()
    from genesis_gb300 import _lib

    gd = np.load(os.path.join(GOLDEN, "substep_small.npz"))
    dt, density, p_size, lx, ly, lz, ux, uy, uz, eps = gd["scene"]
    n = len(gd["in/pos"])
    mats = [material_record(_lib, 0, p[0], p[1], p[2], p[3], p[9], None, p[4], p[5], p[6], p[7], p[8])
            for p in gd["material_params"]]
    c = Ctx([scene_record(_lib, dt, n, (lx, ly, lz), (ux, uy, uz), density, p_size, eps)], mats)
    mat = gd["in/mat"]
    for m in range(len(mats)):
        idx = np.nonzero(mat == m)[0]
        assert np.all(np.diff(idx) == 1)
        c.add(0, 1, int(idx[0]), gd["in/pos"][idx], m)
    yield c, gd, n
    c.close()


def _load(c, gd, n):
    from genesis_gb300 import _lib

    c.set_state(0, 1, pos=gd["in/pos"], vel=gd["in/vel"], C=gd["in/C"], F=gd["in/F"], Jp=gd["in/Jp"],
                active=np.ones(n, np.uint8))
    c.set_field(_lib.FIELD_ACTU, 0, 1, 0, gd["in/actu"][None, :, None])
    c.set_field(_lib.FIELD_MUSCLE_DIR, 0, 1, 0, gd["in/mdir"][None])


def test_first_p2g_grid_matches_reference(ctx):
    c, gd, n = ctx
    _load(c, gd, n)
    c.call("mpm_substep_pre", c.stream)
    g = c.grid(0)
    ref = gd["grid1"]
    assert np.linalg.norm(g[..., 3] - ref[..., 3]) <= 1e-5 * np.linalg.norm(ref[..., 3])
    assert np.linalg.norm(g[..., :3] - ref[..., :3]) <= 1e-5 * np.linalg.norm(ref[..., :3])
    c.call("mpm_substep_grid_op", c.stream)
    c.call("mpm_substep_post", c.stream)
    s = c.get_state(0, 1, n)
    for k, tol in (("pos", 1e-6), ("vel", 1e-4), ("C", 1e-3), ("F", 1e-5), ("Jp", 1e-5)):
        ref = gd["out1/" + k]
        err = np.abs(s[k] - ref).max() / max(1.0, np.abs(ref).max())
        assert err <= tol, (k, err)
    assert c.status()[0] == 0


def test_ten_substeps_match_reference(ctx):
    c, gd, n = ctx
    _load(c, gd, n)
    c.substeps(10)
    s = c.get_state(0, 1, n)
    errs = {}
    for k, tol in (("pos", 1e-5), ("vel", 2e-3), ("C", 2e-2), ("F", 1e-4), ("Jp", 1e-4)):
        ref = gd["out10/" + k]
        errs[k] = np.abs(s[k] - ref).max() / max(1.0, np.abs(ref).max())
        assert errs[k] <= tol, (k, errs[k])
    print("ten-substep golden errors (relative to max):", {k: f"{v:.2e}" for k, v in errs.items()})
    assert c.status()[0] == 0


def test_force_fields_match_reference(ctx):
    """Constant, Wind, Point, Drag, Vortex and Turbulence fields in the CUDA grid op against five
    substeps of the reference's own grid-op and force-field code (tests/golden/force_fields.npz)."""
    from genesis_gb300 import _lib
    from test_golden_oracle import _golden_fields

    c, _, n = ctx
    gf = np.load(os.path.join(GOLDEN, "force_fields.npz"))
    fields = _golden_fields(gf)
    recs = (_lib.MpmForceField * len(fields))(*[f.to_c() for f in fields])
    c.call("mpm_set_force_fields", len(fields), recs)
    try:
        _load(c, gf, n)
        c.substeps(5)
        s = c.get_state(0, 1, n)
        errs = {}
        for k, tol in (("pos", 1e-5), ("vel", 2e-3), ("C", 2e-2), ("F", 1e-4), ("Jp", 1e-4)):
            ref = gf["out5/" + k]
            errs[k] = np.abs(s[k] - ref).max() / max(1.0, np.abs(ref).max())
            assert errs[k] <= tol, (k, errs[k])
        print("force-field golden errors (relative to max):", {k: f"{v:.2e}" for k, v in errs.items()})
        assert c.status()[0] == 0
    finally:
        c.call("mpm_set_force_fields", 0, None)
