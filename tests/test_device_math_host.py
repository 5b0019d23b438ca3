"""The CUDA path's per-particle math (mpm_math.cuh), compiled for the host, against the oracle."""

import ctypes
import os
import subprocess
import tempfile

import numpy as np

import genesis_gb300 as gs
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def shim():
    out = os.path.join(tempfile.mkdtemp(), "libshim.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", os.path.join(HERE, "host_math_shim.cpp"), "-o",
                    out], check=True)
    lib = ctypes.CDLL(out)
    P = ctypes.c_void_p
    lib.shim_svd3_f32.restype = ctypes.c_float
    lib.shim_svd3_f32.argtypes = [P, P, P, P]
    lib.shim_svd3_f64.restype = ctypes.c_double
    lib.shim_svd3_f64.argtypes = [P, P, P, P]
    d = ctypes.c_double
    lib.shim_material_f32.restype = None
    lib.shim_material_f32.argtypes = [ctypes.c_int, ctypes.c_int, d, d, d, d, d, d, d, d, P, ctypes.c_float,
                                      ctypes.c_float, P, ctypes.c_float, P, P, P]
    lib.shim_bspline_w.restype = None
    lib.shim_bspline_w.argtypes = [ctypes.c_float, P]
    return lib


def _svd(lib, A, dtype):
    A = np.ascontiguousarray(A, dtype=dtype)
    U, s, V = np.zeros(9, dtype), np.zeros(3, dtype), np.zeros(9, dtype)
    fn = lib.shim_svd3_f32 if dtype == np.float32 else lib.shim_svd3_f64
    res = fn(A.ctypes.data, U.ctypes.data, s.ctypes.data, V.ctypes.data)
    return U.reshape(3, 3).astype(np.float64), s.astype(np.float64), V.reshape(3, 3).astype(np.float64), res


@pytest.mark.parametrize("scale", [1e-6, 1e-3, 0.1, 1.0])
def test_svd_f32_reconstructs_and_is_rotation_variant(shim, scale):
    rng = np.random.default_rng(1)
    for i in range(2000):
        A = np.eye(3) + scale * rng.normal(size=(3, 3))
        if i % 5 == 0:
            A[:, 2] *= -1  # inverted element
        U, s, V, res = _svd(shim, A.ravel(), np.float32)
        A32 = A.astype(np.float32).astype(np.float64)
        assert np.linalg.norm(U @ np.diag(s) @ V.T - A32) <= 3e-6 * np.linalg.norm(A32)
        assert abs(np.linalg.det(U) - 1) < 1e-5 and abs(np.linalg.det(V) - 1) < 1e-5
        assert s[0] >= -1e-6 and s[1] >= -1e-6
        assert np.sign(s[2]) == np.sign(np.linalg.det(A32)) or abs(s[2]) < 1e-6


def test_svd_exact_identity_and_degenerate(shim):
    for A in (np.eye(3), np.diag([2.0, 2.0, 2.0]), np.diag([1.0, 1.0, 0.0]), np.zeros((3, 3)),
              np.array([[1.0, 1.0, 0.0], [0.0, 0.0, 0.0], [0.0, 0.0, 1.0]])):
        U, s, V, _ = _svd(shim, A.ravel(), np.float32)
        assert np.allclose(U @ np.diag(s) @ V.T, A, atol=1e-6)


def test_svd_matches_oracle_singular_values(shim, oracle):
    rng = np.random.default_rng(2)
    for _ in range(500):
        A = np.eye(3) + 0.3 * rng.normal(size=(3, 3))
        _, s32, _, _ = _svd(shim, A.ravel(), np.float64)
        _, so, _ = oracle.svd(A)
        assert np.allclose(s32, so, rtol=1e-12, atol=1e-12)


def _mat_args(cm):
    mu, lam = cm.mu, cm.lam
    sand_coef = (3 * lam + 2 * mu) / (2 * mu) if mu else 0.0
    vm_ratio = cm.von_mises_yield_stress / (2 * mu) if mu else 0.0
    return (cm.type, cm.flags, mu, lam, cm.friction_alpha, sand_coef, 1 - cm.yield_lower, 1 + cm.yield_higher,
            vm_ratio, cm.stiffness)


MATERIALS = [
    ("Elastic", {}),
    ("Elastic", {"model": "neohooken"}),
    ("Liquid", {}),
    ("Liquid", {"viscous": True}),
    ("Sand", {}),
    ("Snow", {}),
    ("ElastoPlastic", {}),
    ("ElastoPlastic", {"use_von_mises": False}),
    ("Muscle", {}),
]


@pytest.mark.parametrize("name,kw", MATERIALS)
def test_device_material_matches_oracle(shim, oracle, name, kw):
    import genesis_gb300 as gs

    mat = getattr(gs.materials.MPM, name)(**kw)
    cm = mat.to_c(0)
    om = oracle.from_c_material(cm)
    rng = np.random.default_rng(3)
    eps = float(np.finfo(np.float32).eps)
    for i in range(300):
        amp = [1e-3, 3e-2, 0.2][i % 3]
        Ft = (np.eye(3) + amp * rng.normal(size=(3, 3))).astype(np.float32)
        Jp = np.float32(rng.uniform(-0.05, 0.05) if name == "Sand" else rng.uniform(0.9, 1.1))
        actu = np.float32(rng.uniform(0, 1))
        mdir = rng.normal(size=3)
        mdir = (mdir / np.linalg.norm(mdir)).astype(np.float32)
        Fn, jn, P = np.zeros(9, np.float32), np.zeros(1, np.float32), np.zeros(9, np.float32)
        shim.shim_material_f32(*_mat_args(cm), Ft.ctypes.data, float(Jp), float(actu), mdir.ctypes.data, eps,
                               Fn.ctypes.data, jn.ctypes.data, P.ctypes.data)
        Fo, jo, Po = oracle.material_update(om, Ft.astype(np.float64), float(Jp), float(actu), mdir.astype(np.float64))
        # FP32 kernel vs FP64 oracle.  Stress terms like lam*J*(J-1) cancel near J = 1, so the
        # float32 error is relative to the moduli (~eps_f32 * modulus), not to |stress|.
        moduli = abs(cm.lam) + 2 * abs(cm.mu) + cm.stiffness
        hard = np.exp(10 * (1 - jo)) if name == "Snow" else 1.0
        assert np.allclose(Fn.reshape(3, 3), Fo, atol=2e-5 * max(1, np.abs(Fo).max())), (name, i)
        assert abs(jn[0] - jo) <= 2e-5 * max(1.0, abs(jo)), (name, i, jn[0], jo)
        assert np.abs(P.reshape(3, 3) - Po).max() <= 1e-5 * moduli * max(hard, 1.0) + 1e-4 * np.abs(Po).max(), (name, i)


def test_corotated_stress_has_no_rounding_noise_near_identity(shim):
    """F_tmp = I + tiny off-diagonals (as after a free-fall substep): the FP32 stress must be
    of the order of 2 mu |E|, not 2 mu * eps_f32 (noise from degenerate Jacobi rotations)."""
    import genesis_gb300 as gs

    mat = gs.materials.MPM.Elastic(E=3e5, nu=0.2)
    cm = mat.to_c(0)
    rng = np.random.default_rng(5)
    eps = float(np.finfo(np.float32).eps)
    worst = 0.0
    for _ in range(200):
        E = rng.normal(scale=4e-11, size=(3, 3))
        Ft = (np.eye(3) + E).astype(np.float32)
        Fn, jn, P = np.zeros(9, np.float32), np.zeros(1, np.float32), np.zeros(9, np.float32)
        md = np.array([0, 0, 1], np.float32)
        shim.shim_material_f32(*_mat_args(cm), Ft.ctypes.data, 1.0, 0.0, md.ctypes.data, eps, Fn.ctypes.data,
                               jn.ctypes.data, P.ctypes.data)
        worst = max(worst, np.abs(P).max())
    assert worst <= 2 * cm.mu * 1e-9, worst


# ---- known-answer tests from the mathematics of the method (no reference output needed)

def _run_material(shim, cm, Ft, Jp=1.0):
    eps = np.float32(np.finfo(np.float32).eps)
    Ft = np.ascontiguousarray(Ft, np.float32).reshape(9)
    Fn, jn, P = np.zeros(9, np.float32), np.zeros(1, np.float32), np.zeros(9, np.float32)
    md = np.array([0, 0, 1], np.float32)
    shim.shim_material_f32(*_mat_args(cm), Ft.ctypes.data, float(Jp), 0.0, md.ctypes.data, eps, Fn.ctypes.data,
                           jn.ctypes.data, P.ctypes.data)
    return Fn.reshape(3, 3).astype(np.float64), float(jn[0]), P.reshape(3, 3).astype(np.float64)


def test_bspline_partition_of_unity_and_zero_first_moment(shim):
    """Quadratic B-spline weights sum to 1 and sum_o w_o (o - fx) = 0 for fx in [0.5, 1.5)."""
    w = np.zeros(3, np.float32)
    for fx in np.linspace(0.5, 1.5, 41, endpoint=False):
        shim.shim_bspline_w(float(fx), w.ctypes.data)
        assert abs(w.sum() - 1.0) < 1e-6
        assert abs(float(np.dot(w, np.arange(3) - np.float32(fx)))) < 1e-6
        assert np.all(w >= 0)


@pytest.mark.parametrize("name", ["Elastic", "Liquid", "Snow"])
def test_rest_state_has_zero_stress(shim, oracle, name):
    """F = I gives exactly zero stress (corotated: F - UV^T = 0 and J(J - 1) = 0)."""
    cm = getattr(gs.materials.MPM, name)().to_c(0)
    Fn, jn, P = _run_material(shim, cm, np.eye(3))
    assert np.abs(P).max() == 0.0, P
    assert np.allclose(Fn, np.eye(3), atol=1e-7)


def test_sand_expansion_returns_to_identity(shim):
    """Drucker-Prager: a state whose log-strain trace (+ Jp) is non-negative maps to Sigma_new = I
    and Jp_new = trace (sand.py:58-61)."""
    cm = gs.materials.MPM.Sand().to_c(0)
    rng = np.random.default_rng(3)
    for _ in range(20):
        Q1, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        Q2, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        Q1 *= np.sign(np.linalg.det(Q1))
        Q2 *= np.sign(np.linalg.det(Q2))
        sig = rng.uniform(1.01, 1.2, size=3)  # stretched: log strains > 0
        Fn, jn, _ = _run_material(shim, cm, Q1 @ np.diag(sig) @ Q2.T, Jp=0.0)
        R = Q1 @ Q2.T  # U I V^T
        assert np.allclose(Fn, R, atol=2e-5), (Fn, R)
        assert abs(jn - np.log(sig).sum()) < 2e-5


def test_snow_clamps_singular_values(shim):
    """Snow keeps the singular values of F_new inside [1 - 2.5e-2, 1 + 4.5e-3] (snow.py:49-57)."""
    cm = gs.materials.MPM.Snow().to_c(0)
    rng = np.random.default_rng(4)
    for _ in range(20):
        Q1, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        Q2, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        Q1 *= np.sign(np.linalg.det(Q1))
        Q2 *= np.sign(np.linalg.det(Q2))
        sig = rng.uniform(0.9, 1.1, size=3)
        Fn, jn, _ = _run_material(shim, cm, Q1 @ np.diag(sig) @ Q2.T, Jp=1.0)
        s = np.linalg.svd(Fn, compute_uv=False)
        assert s.min() >= 1 - 2.5e-2 - 1e-5 and s.max() <= 1 + 4.5e-3 + 1e-5, s
        clamped = np.clip(sig, 1 - 2.5e-2, 1 + 4.5e-3)
        assert abs(jn - np.prod(sig / clamped)) < 1e-5
