"""Readers of the reference's GEOKERR fixtures (binary layouts of
geokerr_port/validation/gkval_adapters.c:546-555,645-649 and
gkval_io.c:153-166), copied into this folder unchanged.  gkval_manifests/
holds the reference's run manifests (geokerr_port/validation/runs/<ID>/
manifest.json), also unchanged."""
import os
import struct

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read_cache(path=None):
    """GKCH cache file: header (magic, version, S, lam0, dlam, 7 inputs, tpmi, tpri) + 5 x S doubles."""
    path = path or os.path.join(HERE, "geokerr_cache_bfc7797cdaa2b7bb.bin")
    b = open(path, "rb").read()
    magic, ver, S = struct.unpack("<IIQ", b[:16])
    assert magic == 0x474B4348 and ver == 1
    lam0, dlam = struct.unpack("<dd", b[16:32])
    u0, mu0, uf, a, Lz, Q2, t0 = struct.unpack("<7d", b[32:88])
    tpmi, tpri = struct.unpack("<ii", b[88:96])
    body = np.frombuffer(b[96:96 + 40 * S], dtype="<f8").reshape(5, S)
    return dict(S=S, lam0=lam0, dlam=dlam, u0=u0, mu0=mu0, uf=uf, a=a, Lz=Lz, Q2=Q2, t0=t0, tpmi=tpmi, tpri=tpri,
                u=body[0], mu=body[1], t=body[2], phi=body[3], affine=body[4])


def read_fail_window(path):
    """Fail-window file: u32 magic GKPW, u32 version, u16 field, u64 start, end, size; ref[size], port[size]."""
    b = open(path, "rb").read()
    magic, ver = struct.unpack("<II", b[:8])
    assert magic == 0x474B5057
    field, = struct.unpack("<H", b[8:10])
    start, end, size = struct.unpack("<QQQ", b[10:34])
    ref = np.frombuffer(b[34:34 + 8 * size], dtype="<f8")
    port = np.frombuffer(b[34 + 8 * size:34 + 16 * size], dtype="<f8")
    return dict(field=field, start=start, end=end, size=size, ref=ref, port=port)


def fail_windows():
    return sorted(os.path.join(HERE, f) for f in os.listdir(HERE) if f.startswith("geokerr_failwin_"))
