"""ctypes mirror of the POD structs declared in include/np_render.h.

The field order, types and padding follow the C declarations exactly; a
test compares ``ctypes.sizeof`` against the size the library reports.
"""
import ctypes as C

NP_OK = 0
NP_ERR_INVALID = -1
NP_ERR_ALLOC = -2
NP_ERR_KERNEL = -3
NP_ERR_NO_DEVICE = -4
NP_ERR_TIMEOUT = -5

NP_UNITS_RS, NP_UNITS_M = 0, 1
NP_JITTER_WANGHASH, NP_JITTER_STRATIFIED, NP_JITTER_CRITICAL = 0, 1, 2
NP_CAMERA_STATIC, NP_CAMERA_ZAMO = 0, 1
NP_INTEG_RK4, NP_INTEG_ADAPTIVE, NP_INTEG_RKF78 = 0, 1, 2
NP_CROSS_LINEAR, NP_CROSS_HERMITE, NP_CROSS_ROOT = 0, 1, 2
NP_BG_GRADIENT, NP_BG_POINT = 0, 1
NP_PREC_FP64, NP_PREC_MIXED = 0, 1
NP_ISLAND_HORIZON, NP_ISLAND_TURNING, NP_ISLAND_CRITICAL = 1, 2, 4
NP_ISLANDS_ALL = 7
NP_ISLANDS_DEFAULT = NP_ISLAND_HORIZON | NP_ISLAND_CRITICAL
NP_ISLAND_ARITH_FP64, NP_ISLAND_ARITH_DF = 0, 1
NP_CRITICAL_CLOSED_FORM, NP_CRITICAL_INTEGRATE = 0, 1


class Scene(C.Structure):
    """np_scene_t (include/np_render.h)."""
    _fields_ = [
        ("width", C.c_int32), ("height", C.c_int32),
        ("spp", C.c_int32), ("sample_offset", C.c_int32),
        ("mass", C.c_double), ("spin", C.c_double), ("r_cam", C.c_double),
        ("theta_deg", C.c_double), ("phi_deg", C.c_double), ("fov_y_deg", C.c_double),
        ("units", C.c_int32), ("camera", C.c_int32),
        ("jitter", C.c_int32), ("seed", C.c_uint32),
        ("integrator", C.c_int32), ("max_steps", C.c_int32),
        ("step_scale", C.c_double), ("rtol", C.c_double), ("atol", C.c_double),
        ("escape_r", C.c_double),
        ("disk_on", C.c_int32), ("disk_max_orders", C.c_int32),
        ("disk_rin", C.c_double), ("disk_rout", C.c_double),
        ("emissivity_q", C.c_double), ("disk_gain", C.c_double),
        ("crossing", C.c_int32), ("background", C.c_int32),
        ("bg_sigma_deg", C.c_double), ("bg_brightness", C.c_double),
        ("check_invariants", C.c_int32), ("islands", C.c_int32),
        ("inv_gate", C.c_double), ("rtol_fp64", C.c_double),
        ("island_arith", C.c_int32), ("critical_solver", C.c_int32),
    ]

    def copy(self):
        s = Scene()
        C.memmove(C.byref(s), C.byref(self), C.sizeof(Scene))
        return s

    def replace(self, **kw):
        s = self.copy()
        for k, v in kw.items():
            if not hasattr(s, k):
                raise AttributeError(k)
            setattr(s, k, v)
        return s


class RenderStats(C.Structure):
    """np_render_stats_t (include/np_render.h)."""
    _fields_ = [
        ("rays", C.c_uint64), ("steps", C.c_uint64), ("fp64_steps", C.c_uint64),
        ("rhs_evals", C.c_uint64), ("deferred_rays", C.c_uint64),
        ("kernel_ms", C.c_double), ("init_ms", C.c_double), ("closed_form_rays", C.c_uint64), ("band_rays", C.c_uint64),
    ]


def isco_radius(mass, spin):
    """Prograde ISCO radius (Bardeen, Press & Teukolsky 1972), in the units of ``mass``."""
    import math
    a = spin
    z1 = 1.0 + math.cbrt(1.0 - a * a) * (math.cbrt(1.0 + a) + math.cbrt(1.0 - a))
    z2 = math.sqrt(3.0 * a * a + z1 * z1)
    sgn = 1.0 if a >= 0 else -1.0
    return mass * (3.0 + z2 - sgn * math.sqrt((3.0 - z1) * (3.0 + z1 + 2.0 * z2)))


def reference_defaults():
    """render.cu:15-46 defaults (lengths in Rs, wanghash jitter, FP64 RK4)."""
    return Scene(width=1280, height=720, spp=1, sample_offset=0,
                 mass=10.0, spin=0.0, r_cam=50.0, theta_deg=90.0, phi_deg=0.0, fov_y_deg=50.0,
                 units=NP_UNITS_RS, camera=NP_CAMERA_STATIC, jitter=NP_JITTER_WANGHASH, seed=0,
                 integrator=NP_INTEG_RK4, max_steps=10000, step_scale=0.01,
                 rtol=1e-10, atol=1e-12, escape_r=0.0,
                 disk_on=1, disk_max_orders=1, disk_rin=0.0, disk_rout=0.0,
                 emissivity_q=2.0, disk_gain=1.0, crossing=NP_CROSS_LINEAR,
                 background=NP_BG_GRADIENT, bg_sigma_deg=1.0, bg_brightness=3.0,
                 check_invariants=0, islands=NP_ISLANDS_DEFAULT, inv_gate=0.0, rtol_fp64=0.0, island_arith=NP_ISLAND_ARITH_FP64, critical_solver=NP_CRITICAL_CLOSED_FORM)


def benchmark_scene(width=1280, height=720, spp=4, spin=0.9, seed=0):
    """The 1280x720, a=0.9 Kerr scene: M=1, r_cam=50 M, theta=80 deg, fov 55 deg,
    stratified jitter, disk ISCO..20 M with j ~ r^-3, 3 orders, step cap 4096,
    escape at 1000 M, cubic-Hermite crossing location."""
    return Scene(width=width, height=height, spp=spp, sample_offset=0,
                 mass=1.0, spin=spin, r_cam=50.0, theta_deg=80.0, phi_deg=0.0, fov_y_deg=55.0,
                 units=NP_UNITS_M, camera=NP_CAMERA_STATIC, jitter=NP_JITTER_STRATIFIED, seed=seed,
                 integrator=NP_INTEG_RK4, max_steps=4096, step_scale=0.01,
                 rtol=1e-7, atol=1e-12, escape_r=1000.0,
                 disk_on=1, disk_max_orders=3, disk_rin=isco_radius(1.0, spin), disk_rout=20.0,
                 emissivity_q=3.0, disk_gain=1.0, crossing=NP_CROSS_HERMITE,
                 background=NP_BG_GRADIENT, bg_sigma_deg=1.0, bg_brightness=3.0,
                 check_invariants=0, islands=NP_ISLANDS_DEFAULT, inv_gate=0.0, rtol_fp64=0.0, island_arith=NP_ISLAND_ARITH_FP64, critical_solver=NP_CRITICAL_CLOSED_FORM)


def accurate_scene(scene, rtol=1e-8, atol=1e-9, islands=None):
    """`scene` on the mixed path's embedded 7(8) integrator: compensated FP32
    steps under error control at `rtol` / `atol`, crossings landed on the
    equator by a Henon step, FP64 islands at rtol, near-critical and
    horizon-band rays in FP64 closed form.  At the
    defaults the first disk crossing of the 1280x720x4, a = 0.9 benchmark
    frame is within 1e-5 M of the Mino-time solver's (p99).  Render it with
    precision "mixed"."""
    kw = dict(integrator=NP_INTEG_RKF78, crossing=NP_CROSS_ROOT, rtol=rtol, atol=atol)
    if islands is not None:
        kw["islands"] = islands
    return scene.replace(**kw)


def research_scene(scene, rtol=1e-12, atol=1e-14, inv_gate=1e-12):
    """`scene` in research mode, as the CLI's --mode research sets it: the
    embedded 7(8) integrator at tight tolerances, root-found crossings, the
    invariant gate, the ZAMO camera and invariant tracking.  Render it with
    precision "fp64"."""
    return scene.replace(integrator=NP_INTEG_RKF78, crossing=NP_CROSS_ROOT, rtol=rtol, atol=atol,
                         inv_gate=inv_gate, camera=NP_CAMERA_ZAMO, check_invariants=1)
