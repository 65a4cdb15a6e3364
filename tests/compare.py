"""Field-by-field comparison of two exported world states (dbox_gb300.abi records)."""
import numpy as np

# b2Contact flag bits compared bit-exactly; island (1) and toi (0x20) are solver-internal marks
CONTACT_FLAG_MASK = 0x2 | 0x4 | 0x8 | 0x10


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _rows(x, y):
    """Per-row 'bits differ' of two equally shaped record fields (works for empty arrays)."""
    d = _bits(x) != _bits(y)
    return d.reshape(d.shape[0], int(np.prod(d.shape[1:]))).any(1) if d.ndim > 1 else d


def exact_diff(a, b):
    """Names of fields whose bit patterns differ (state dicts from export_state)."""
    out = []
    ha, hb = a["header"][0], b["header"][0]
    for f in ("body_count", "fixture_count", "contact_count", "joint_count", "step_complete"):
        if ha[f] != hb[f]:
            out.append("header.%s %s != %s" % (f, ha[f], hb[f]))
    if _bits(np.float32(ha["inv_dt0"])) != _bits(np.float32(hb["inv_dt0"])):
        out.append("header.inv_dt0")
    if out:
        return out
    ba, bb = a["bodies"], b["bodies"]
    for f in ("flags", "type"):
        bad = np.nonzero(ba[f] != bb[f])[0]
        if len(bad):
            out.append("bodies.%s at %s" % (f, bad[:8].tolist()))
    for f in ("xf", "sweep", "vel", "force", "sleep_time", "mass"):
        bad = np.nonzero(_rows(ba[f], bb[f]))[0]
        if len(bad):
            out.append("bodies.%s at %s" % (f, bad[:8].tolist()))
    pa, pb = a["proxies"], b["proxies"]
    for f in ("moved", "proxy_id"):
        bad = np.nonzero(pa[f] != pb[f])[0]
        if len(bad):
            out.append("proxies.%s at %s" % (f, bad[:8].tolist()))
    d = _rows(pa["fat_aabb"], pb["fat_aabb"])
    if d.any():
        out.append("proxies.fat_aabb at %s" % np.nonzero(d)[0][:8].tolist())
    ca, cb = a["contacts"], b["contacts"]
    for f in ("fixture_a", "fixture_b", "toi_count", "point_count", "type"):
        bad = np.nonzero(ca[f] != cb[f])[0]
        if len(bad):
            out.append("contacts.%s at %s" % (f, bad[:8].tolist()))
            return out
    bad = np.nonzero((ca["flags"] & CONTACT_FLAG_MASK) != (cb["flags"] & CONTACT_FLAG_MASK))[0]
    if len(bad):
        out.append("contacts.flags at %s" % bad[:8].tolist())
    for f in ("friction", "restitution", "tangent_speed", "local_normal", "local_point"):
        d = _rows(ca[f], cb[f])
        # a manifold with no points carries stale normal/point data; compare only touching ones
        if f in ("local_normal", "local_point"):
            d &= ca["point_count"] > 0
        bad = np.nonzero(d)[0]
        if len(bad):
            out.append("contacts.%s at %s" % (f, bad[:8].tolist()))
    for k in range(2):
        live = ca["point_count"] > k
        for f in ("local_point", "normal_impulse", "tangent_impulse", "id"):
            bad = np.nonzero(_rows(ca["points"][f][:, k], cb["points"][f][:, k]) & live)[0]
            if len(bad):
                out.append("contacts.points[%d].%s at %s" % (k, f, bad[:8].tolist()))
    ja, jb = a["joints"], b["joints"]
    if len(ja):
        d = _rows(ja["impulse"], jb["impulse"])
        if d.any():
            out.append("joints.impulse at %s" % np.nonzero(d)[0][:8].tolist())
    return out


def structure_diff(a, b):
    """Pair set, contact list order, manifold point counts and feature ids (the bit-exact set)."""
    out = []
    ca, cb = a["contacts"], b["contacts"]
    if len(ca) != len(cb):
        return ["contact count %d != %d" % (len(ca), len(cb))]
    for f in ("fixture_a", "fixture_b", "point_count"):
        bad = np.nonzero(ca[f] != cb[f])[0]
        if len(bad):
            out.append("contacts.%s at %s" % (f, bad[:8].tolist()))
    if out:
        return out
    for k in range(2):
        live = ca["point_count"] > k
        bad = np.nonzero((ca["points"]["id"][:, k] != cb["points"]["id"][:, k]) & live)[0]
        if len(bad):
            out.append("contacts.points[%d].id at %s" % (k, bad[:8].tolist()))
    bad = np.nonzero((ca["flags"] & 0x6) != (cb["flags"] & 0x6))[0]
    if len(bad):
        out.append("contacts.touching/enabled at %s" % bad[:8].tolist())
    return out


def body_error(a, b):
    """Max |difference| of position (m), angle (rad) and velocity (m/s) over bodies."""
    ba, bb = a["bodies"], b["bodies"]
    dp = float(np.abs(ba["xf"][:, :2].astype(np.float64) - bb["xf"][:, :2]).max()) if len(ba) else 0.0
    da = float(np.abs(ba["sweep"][:, 7].astype(np.float64) - bb["sweep"][:, 7]).max()) if len(ba) else 0.0
    dv = float(np.abs(ba["vel"][:, :2].astype(np.float64) - bb["vel"][:, :2]).max()) if len(ba) else 0.0
    dw = float(np.abs(ba["vel"][:, 2].astype(np.float64) - bb["vel"][:, 2]).max()) if len(ba) else 0.0
    return dp, da, max(dv, dw)
