"""Batched scenes over the np_batch_* C ABI (include/np_render.h).

    scenes = uneven_scenes(256, seed=1)
    b = Batch(scenes)
    autotune(Batch(scenes[::8]))          # tune on a sub-batch, installs the best setting
    st = b.run(graph=True, stats=True)    # one persistent launch, replayed as a CUDA graph
    rgb, rc = b.image(17)

The batch traces every scene with the mixed-precision path in one launch
over a single device ray queue.
"""
import ctypes as C

import numpy as np

from ._abi import Scene, benchmark_scene, isco_radius, NP_PREC_MIXED
from ._lib import load, check


class BatchStats(C.Structure):
    """np_batch_stats_t."""
    _fields_ = [("scenes", C.c_int32), ("rays", C.c_uint64), ("steps", C.c_uint64), ("fp64_steps", C.c_uint64),
                ("deferred_rays", C.c_uint64), ("total_ms", C.c_double), ("scene_ms_p50", C.c_double),
                ("scene_ms_p99", C.c_double), ("scene_ms_max", C.c_double), ("block", C.c_int32),
                ("min_blocks", C.c_int32), ("chunk", C.c_int32), ("island_batch", C.c_int32),
                ("closed_form_rays", C.c_uint64)]

    def as_dict(self):
        return {f[0]: getattr(self, f[0]) for f in self._fields_}


class BatchTune(C.Structure):
    """np_batch_tune_t."""
    _fields_ = [("shape", C.c_int32), ("block", C.c_int32), ("min_blocks", C.c_int32), ("chunk", C.c_int32),
                ("island_batch", C.c_int32), ("trials", C.c_int32), ("best_ms", C.c_double)]

    def as_dict(self):
        return {f[0]: getattr(self, f[0]) for f in self._fields_}


_PROTOS = {
    "np_batch_create": (C.c_void_p, [C.POINTER(Scene), C.c_int, C.c_int, C.c_void_p]),
    "np_batch_destroy": (None, [C.c_void_p]),
    "np_batch_run": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(BatchStats)]),
    "np_batch_scene_output": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
    "np_batch_copy_output": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "np_batch_scene_latency": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "np_batch_set_tuning": (C.c_int, [C.c_int, C.c_int, C.c_int]),
    "np_batch_shape": (C.c_int, [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "np_batch_autotune": (C.c_int, [C.c_void_p, C.POINTER(BatchTune)]),
}


def _lib():
    lib = load()
    if not getattr(lib, "_batch_ready", False):
        for name, (res, args) in _PROTOS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        lib._batch_ready = True
    return lib


RESOLUTIONS = (64, 128, 256, 512)


def uneven_scenes(n=256, seed=1):
    """The uneven-batch workload: n benchmark-type scenes (r_cam 50 M, fov
    55 deg, disk ISCO..20 M with j ~ r^-3, step cap 4096, escape 1000 M) with
    spin ~ U[0, 0.998], inclination ~ U[5, 85] deg, square resolution drawn
    from {64, 128, 256, 512}, 1..8 spp and 1..3 disk orders, all from one
    numpy generator seeded with `seed`."""
    rng = np.random.default_rng(seed)
    spin = rng.uniform(0.0, 0.998, n)
    incl = rng.uniform(5.0, 85.0, n)
    res = rng.choice(np.array(RESOLUTIONS), n)
    spp = rng.integers(1, 9, n)
    orders = rng.integers(1, 4, n)
    out = []
    for i in range(n):
        sc = benchmark_scene(width=int(res[i]), height=int(res[i]), spp=int(spp[i]), spin=float(spin[i]), seed=seed)
        out.append(sc.replace(theta_deg=float(incl[i]), disk_max_orders=int(orders[i]),
                              disk_rin=isco_radius(1.0, float(spin[i]))))
    return out


class Batch:
    """Device-resident batch of scenes (np_batch_t)."""

    def __init__(self, scenes, stream=None):
        import torch
        self.lib = _lib()
        self.scenes = list(scenes)
        arr = (Scene * len(self.scenes))(*self.scenes)
        self.stream = stream if stream is not None else torch.cuda.current_stream()
        self.h = self.lib.np_batch_create(arr, len(self.scenes), NP_PREC_MIXED, C.c_void_p(self.stream.cuda_stream))
        if not self.h:
            check(-1)

    @property
    def rays(self):
        return sum(s.width * s.height * s.spp for s in self.scenes)

    def run(self, graph=True, stats=False):
        st = BatchStats() if stats else None
        check(self.lib.np_batch_run(self.h, 1 if graph else 0, C.byref(st) if st is not None else None))
        return st

    def image(self, i):
        """(rgb [3, H, W], rcross [H, W]) of scene i from the last pass, copied
        into new CUDA tensors."""
        import torch
        sc = self.scenes[i]
        rgb = torch.empty((3, sc.height, sc.width), dtype=torch.float32, device="cuda")
        rc = torch.empty((sc.height, sc.width), dtype=torch.float32, device="cuda")
        check(self.lib.np_batch_copy_output(self.h, i, C.c_void_p(rgb.data_ptr()), C.c_void_p(rc.data_ptr())))
        self.stream.synchronize()
        return rgb, rc

    def latency_ms(self):
        out = (C.c_double * len(self.scenes))()
        check(self.lib.np_batch_scene_latency(self.h, out))
        return np.array(out[:])

    def close(self):
        if self.h:
            self.lib.np_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune(batch):
    """Runs the library's autotuner on `batch` and returns the chosen setting."""
    t = BatchTune()
    check(_lib().np_batch_autotune(batch.h, C.byref(t)))
    return t.as_dict()


def set_tuning(shape=0, chunk=64, island_batch=8):
    check(_lib().np_batch_set_tuning(shape, chunk, island_batch))
