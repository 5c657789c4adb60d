"""Reader of Houdini's classic binary geometry files (.bgeo, format version 5, the layout partio writes and reads),
written from the format's description for the tests: big-endian header (magic "Bgeo", 'V', version, eight
int32 counts), the point attributes' names, sizes, types and defaults, one record per point (x, y, z, w and the
attributes' values), then the end bytes 0x00 0xff. Only point attributes of float (0) and vector (5) type."""
import struct

import numpy as np


def read_bgeo(path):
    with open(path, "rb") as f:
        buf = f.read()
    if buf[:4] != b"Bgeo" or buf[4:5] != b"V":
        raise ValueError("not a binary geometry file")
    (version,) = struct.unpack(">i", buf[5:9])
    counts = struct.unpack(">8i", buf[9:41])
    n_points, n_prims, n_pgroups, n_primgroups, n_pattr, n_vattr, n_primattr, n_detail = counts
    if version != 5 or n_prims or n_pgroups or n_primgroups or n_vattr or n_primattr or n_detail:
        raise ValueError("only points with point attributes are read")
    pos = 41
    attrs = []
    for _ in range(n_pattr):
        (ln,) = struct.unpack(">H", buf[pos:pos + 2])
        name = buf[pos + 2:pos + 2 + ln].decode()
        pos += 2 + ln
        size, typ = struct.unpack(">Hi", buf[pos:pos + 6])
        pos += 6
        if typ not in (0, 5):
            raise ValueError(f"attribute {name}: type {typ}")
        pos += 4 * size  # defaults
        attrs.append((name, size))
    per = 4 + sum(sz for _, sz in attrs)
    rec = np.frombuffer(buf, dtype=">f4", count=n_points * per, offset=pos).reshape(n_points, per).astype(np.float64)
    pos += 4 * n_points * per
    if buf[pos:] != b"\x00\xff":
        raise ValueError("missing end bytes")
    out = {"P": rec[:, :3], "w": rec[:, 3]}
    c = 4
    for name, size in attrs:
        out[name] = rec[:, c:c + size] if size > 1 else rec[:, c]
        c += size
    return out
