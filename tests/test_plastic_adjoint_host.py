"""The Sand, Snow and ElastoPlastic adjoints of the differentiable substep
(genesis_gb300/csrc/mpm_adjoint.cuh), compiled for the host, against FP64 central differences of the
same material update (material_update, the code the kernels run): dL/dF_tmp and dL/dJp for
L = <gFn, F_new> + <gP, P> + gJpn Jp_new with random weights, in every regime of the laws
(Sand: expanding tr >= 0, compressed and elastic (dg <= 0), compressed and yielding; Snow and the
clamped ElastoPlastic: inside the clamp, stretched past the upper bound, compressed past the lower
bound; von Mises ElastoPlastic: below and past the yield surface), including F_tmp = I and nearly
coinciding singular values."""

import ctypes
import math
import os
import subprocess
import tempfile

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
EPS32 = float(np.finfo(np.float32).eps)
MT_SAND, MT_SNOW, MT_ELASTOPLASTIC = 2, 3, 4
EP_VON_MISES = 64 + MT_ELASTOPLASTIC  # the von Mises law's id in mpm_adjoint.cuh
KINDS = [MT_SAND, MT_SNOW, MT_ELASTOPLASTIC, EP_VON_MISES]


@pytest.fixture(scope="module")
def shim():
    out = os.path.join(tempfile.mkdtemp(), "libshim.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", os.path.join(HERE, "host_math_shim.cpp"), "-o",
                    out], check=True)
    lib = ctypes.CDLL(out)
    P, d = ctypes.c_void_p, ctypes.c_double
    lib.shim_plastic_forward_f64.argtypes = [ctypes.c_int, d, d, d, d, d, P, d, P, P, P]
    lib.shim_plastic_adjoint_f64.argtypes = [ctypes.c_int, d, d, d, d, d, P, d, P, P, d, P, P, P, P]
    lib.shim_plastic_adjoint_f32.argtypes = [ctypes.c_int, d, d, d, d, ctypes.c_float, P, ctypes.c_float, P, P,
                                             ctypes.c_float, P, P]
    return lib


def _params(kind):
    E, nu = {MT_SAND: (1e6, 0.2), MT_SNOW: (1.4e5, 0.2)}.get(kind, (3e5, 0.2))
    mu, lam = E / (2 * (1 + nu)), E * nu / ((1 + nu) * (1 - 2 * nu))
    if kind == MT_SAND:
        s = math.sin(math.radians(45.0))
        return mu, lam, math.sqrt(2 / 3) * 2 * s / (3 - s), 0.0
    if kind == EP_VON_MISES:
        return mu, lam, 1e4 / (2 * mu), 0.0  # von_mises_yield_stress 1e4
    return mu, lam, 1 - 2.5e-2, 1 + 4.5e-3


def _forward(lib, kind, Ft, Jp):
    mu, lam, p0, p1 = [float(np.float32(v)) for v in _params(kind)]
    Ft = np.ascontiguousarray(Ft, np.float64)
    Fn, P, jn = np.zeros(9), np.zeros(9), ctypes.c_double()
    lib.shim_plastic_forward_f64(kind, mu, lam, p0, p1, EPS32, Ft.ctypes.data, Jp, Fn.ctypes.data,
                                 ctypes.byref(jn), P.ctypes.data)
    return Fn, jn.value, P


def _regime(kind, Ft, Jp):
    s = np.linalg.svd(Ft.reshape(3, 3), compute_uv=False)
    if kind in (MT_SNOW, MT_ELASTOPLASTIC):
        return tuple(int(v < 1 - 2.5e-2) - int(v > 1 + 4.5e-3) for v in s)
    if kind == EP_VON_MISES:
        e = np.log(np.maximum(s, 0.05))
        eh = e - e.mean()
        return (int(math.sqrt((eh ** 2).sum() + EPS32) - _params(kind)[2] > 0),)
    e = np.log(np.maximum(np.abs(s), 1e-4))
    tr = e.sum() + Jp
    if tr >= 0:
        return (0,)
    mu, lam, alpha, _ = _params(kind)
    eh = e - tr / 3
    dg = math.sqrt((eh ** 2).sum() + EPS32) + (3 * lam + 2 * mu) / (2 * mu) * tr * alpha
    return (1, int(dg > 0))


def _cases(kind, rng):
    out = [(np.eye(3), 0.0 if kind == MT_SAND else 1.0)]
    for i in range(40):
        amp = [1e-4, 3e-3, 2e-2, 0.1][i % 4]
        Ft = np.eye(3) + amp * rng.normal(size=(3, 3))
        if i % 7 == 3:  # two nearly coinciding singular values
            U, _, Vt = np.linalg.svd(rng.normal(size=(3, 3)))
            Ft = U @ np.diag([1.0 + amp, 1.0 + amp * (1 + 1e-6), 1.0 - amp]) @ Vt
            if np.linalg.det(Ft) < 0:
                Ft = -Ft
        if kind == MT_SAND:
            Jp = rng.choice([0.0, rng.uniform(-0.05, 0.05)])
        elif kind == MT_SNOW:
            Jp = rng.uniform(0.9, 1.1)
        else:
            Jp = 1.0
        out.append((Ft, Jp))
    return out


@pytest.mark.parametrize("kind", KINDS)
def test_plastic_adjoint_matches_fp64_central_differences(shim, kind):
    rng = np.random.default_rng(7 + kind)
    seen = set()
    for Ft, Jp in _cases(kind, rng):
        gFn, gP, gJpn = rng.normal(size=9), rng.normal(size=9) * 1e-5, rng.normal()
        mu, lam, p0, p1 = [float(np.float32(v)) for v in _params(kind)]

        def L(F, J):
            Fn, jn, P = _forward(shim, kind, F, J)
            return gFn @ Fn + gP @ P + gJpn * jn

        gFt, gJp, gmu, glam = np.zeros(9), ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        Fr = np.ascontiguousarray(Ft.reshape(-1), np.float64)
        shim.shim_plastic_adjoint_f64(kind, mu, lam, p0, p1, EPS32, Fr.ctypes.data, Jp, gFn.ctypes.data,
                                      gP.ctypes.data, gJpn, gFt.ctypes.data, ctypes.byref(gJp), ctypes.byref(gmu),
                                      ctypes.byref(glam))
        h = 1e-7
        reg = _regime(kind, Fr, Jp)
        fd = np.zeros(9)
        ok = True
        for k in range(9):
            e = np.zeros(9)
            e[k] = h
            if _regime(kind, Fr + e, Jp) != reg or _regime(kind, Fr - e, Jp) != reg:
                ok = False  # a finite difference across a yield surface measures the kink, not the derivative
                break
            fd[k] = (L(Fr + e, Jp) - L(Fr - e, Jp)) / (2 * h)
        if not ok:
            continue
        seen.add(reg)
        scale = max(np.abs(fd).max(), 1e-12)
        assert np.abs(gFt - fd).max() <= 2e-5 * scale + 1e-9, (reg, gFt, fd)
        if _regime(kind, Fr, Jp + h) == reg and _regime(kind, Fr, Jp - h) == reg:
            fj = (L(Fr, Jp + h) - L(Fr, Jp - h)) / (2 * h)
            assert abs(gJp.value - fj) <= 2e-5 * max(abs(fj), scale) + 1e-9, (reg, gJp.value, fj)
    want = {MT_SAND: {(0,), (1, 0), (1, 1)}, EP_VON_MISES: {(0,), (1,)}}.get(kind, {(0, 0, 0)})
    assert want <= seen, seen
    if kind in (MT_SNOW, MT_ELASTOPLASTIC):
        assert any(r != (0, 0, 0) for r in seen), seen


@pytest.mark.parametrize("kind", KINDS)
def test_plastic_adjoint_float_close_to_double(shim, kind):
    """The float build the kernel runs stays within float rounding of the double one, F = I included."""
    rng = np.random.default_rng(3)
    for Ft, Jp in _cases(kind, rng)[:12]:
        gFn, gP, gJpn = rng.normal(size=9), rng.normal(size=9) * 1e-5, rng.normal()
        mu, lam, p0, p1 = _params(kind)
        Fr = np.ascontiguousarray(Ft.reshape(-1), np.float64)
        g64 = np.zeros(9)
        j64, m64, l64 = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        shim.shim_plastic_adjoint_f64(kind, mu, lam, p0, p1, EPS32, Fr.ctypes.data, Jp, gFn.ctypes.data,
                                      gP.ctypes.data, gJpn, g64.ctypes.data, ctypes.byref(j64), ctypes.byref(m64),
                                      ctypes.byref(l64))
        F32 = Fr.astype(np.float32)
        gFn32, gP32 = gFn.astype(np.float32), gP.astype(np.float32)  # kept alive through the call
        g32 = np.zeros(9, np.float32)
        j32 = ctypes.c_float()
        shim.shim_plastic_adjoint_f32(kind, mu, lam, p0, p1, EPS32, F32.ctypes.data, Jp, gFn32.ctypes.data,
                                      gP32.ctypes.data, gJpn, g32.ctypes.data, ctypes.byref(j32))
        assert np.all(np.isfinite(g32))
        assert np.abs(g32 - g64).max() <= 2e-3 * max(np.abs(g64).max(), 1.0), (g32, g64)
