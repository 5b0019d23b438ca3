"""Build libgbmpm contexts directly through the C ABI (used by GPU tests)."""

import ctypes

import numpy as np
import torch


def material_record(lib_mod, scene, t, flags, mu, lam, rho=1000.0, default_Jp=None, alpha=0.0, yl=0.0, yh=0.0, vm=0.0,
                    stiffness=0.0):
    m = lib_mod.MpmMaterial()
    m.type, m.flags, m.scene = int(t), int(flags), int(scene)
    m.mu, m.lam, m.rho = float(mu), float(lam), float(rho)
    m.default_Jp = float((0.0 if int(t) == 2 else 1.0) if default_Jp is None else default_Jp)
    m.friction_alpha, m.yield_lower, m.yield_higher = float(alpha), float(yl), float(yh)
    m.von_mises_yield_stress, m.stiffness = float(vm), float(stiffness)
    return m


def scene_record(lib_mod, dt, n, lower=(0, 0, 0), upper=(1, 1, 1), density=64.0, p_size=None, eps=None,
                 gravity=(0.0, 0.0, -9.81)):
    c = lib_mod.MpmSceneConfig()
    c.substep_dt = dt
    for d in range(3):
        c.gravity[d], c.lower_bound[d], c.upper_bound[d] = gravity[d], lower[d], upper[d]
    c.grid_density = density
    c.particle_size = p_size if p_size is not None else 0.01 * 64.0 / density
    c.mass_eps = eps if eps is not None else float(np.finfo(np.float32).eps)
    c.restitution = 0.0
    c.n_particles = int(n)
    return c


class Ctx:
    def __init__(self, scenes, materials):
        from genesis_gb300 import _lib

        self.m = _lib
        self.lib = _lib.load()
        S = (_lib.MpmSceneConfig * len(scenes))(*scenes)
        M = (_lib.MpmMaterial * len(materials))(*materials)
        self.ctx = ctypes.c_void_p()
        _lib.check(self.lib.mpm_ctx_create(S, len(scenes), M, len(materials), torch.cuda.current_device(),
                                           ctypes.byref(self.ctx)), None, "create")
        self.n_scenes = len(scenes)

    @property
    def stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def call(self, name, *args):
        self.m.check(getattr(self.lib, name)(self.ctx, *args), self.ctx, name)

    def add(self, s0, s1, start, pos, mat, active=1):
        p = torch.as_tensor(np.asarray(pos, np.float32), device="cuda").contiguous()
        self.call("mpm_add_particles", s0, s1, start, len(p), mat, active, p.data_ptr(), self.stream)
        torch.cuda.synchronize()

    def set_state(self, s0, s1, **kw):
        t = {k: (None if kw.get(k) is None else torch.as_tensor(np.asarray(kw[k]), device="cuda").contiguous())
             for k in ("pos", "vel", "C", "F", "Jp", "active")}
        t = {k: (None if v is None else (v.to(torch.uint8) if k == "active" else v.float())) for k, v in t.items()}
        ptrs = [None if t[k] is None else t[k].data_ptr() for k in ("pos", "vel", "C", "F", "Jp", "active")]
        self.call("mpm_set_state", s0, s1, *ptrs, self.stream)
        torch.cuda.synchronize()

    def get_state(self, s0, s1, n_total):
        out = dict(pos=torch.empty(n_total, 3), vel=torch.empty(n_total, 3), C=torch.empty(n_total, 3, 3),
                   F=torch.empty(n_total, 3, 3), Jp=torch.empty(n_total), active=torch.empty(n_total, dtype=torch.uint8))
        out = {k: v.cuda() for k, v in out.items()}
        self.call("mpm_get_state", s0, s1, *[out[k].data_ptr() for k in ("pos", "vel", "C", "F", "Jp", "active")],
                  self.stream)
        torch.cuda.synchronize()
        return {k: v.cpu().numpy() for k, v in out.items()}

    def set_field(self, field, s0, s1, start, data):
        d = torch.as_tensor(np.asarray(data, np.float32), device="cuda").contiguous()
        self.call("mpm_set_particles", field, s0, s1, start, d.shape[1], d.data_ptr(), self.stream)
        torch.cuda.synchronize()

    def grid(self, scene):
        res = (ctypes.c_int32 * 3)()
        self.lib.mpm_scene_grid_res(self.ctx, scene, res)
        out = torch.empty((res[0], res[1], res[2], 4), device="cuda")
        self.call("mpm_get_grid", scene, out.data_ptr(), self.stream)
        torch.cuda.synchronize()
        return out.double().cpu().numpy()

    def substeps(self, n):
        self.call("mpm_substeps", n, self.stream)

    def status(self):
        st, f64 = ctypes.c_uint32(), ctypes.c_int64()
        self.call("mpm_status_word", ctypes.byref(st), ctypes.byref(f64), 1, self.stream)
        return st.value, f64.value

    def close(self):
        if self.ctx:
            self.lib.mpm_ctx_destroy(self.ctx)
            self.ctx = None
