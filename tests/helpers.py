"""Small shared helpers for the test suite."""
import numpy as np


def rel(a, b):
    """max |a - b| / max |b| (0 if both vanish)."""
    a, b = np.asarray(a), np.asarray(b)
    d = np.abs(a - b).max()
    s = np.abs(b).max()
    return 0.0 if d == 0 else d / (s if s > 0 else 1.0)


def rand_spec(T, nb, seed=1, slope=0.0):
    from gdpy import inputs

    rng = np.random.default_rng(seed)
    deg, order = inputs.degree_order(T)
    a = rng.standard_normal((nb, deg.size)) + 1j * rng.standard_normal((nb, deg.size))
    a[:, order == 0] = a[:, order == 0].real
    if slope:
        a *= np.maximum(deg, 1).astype(float) ** slope
    return a


def sig_to_dict(h):
    """A gdpy.sigio.SigHead as the header dict of the sigma-file oracle."""
    import sigio_oracle as so

    d = so.default_head()
    d["clabsig"] = h.label
    d["fhour"] = h.fhour
    d["idate"] = list(h.idate)
    for k in ("si", "sl", "ak", "bk"):
        d[k] = np.ctypeslib.as_array(getattr(h, k)).astype(np.float32).copy()
    for k in so.INT_FIELDS:
        d[k] = getattr(h, k) if not k.startswith("iens") else h.iens[int(k[-1])]
    for k in ("pdryini", "ncldt", "ixgr", "ivs", "nxgr", "nxss", "nhead", "ndata"):
        d[k] = getattr(h, k)
    d["vcoord"] = h.vcoord_array
    d["cfvars"] = h.cfvar_names
    n = h.ntrac + 1
    d["cpi"] = np.ctypeslib.as_array(h.cpi)[:n].copy()
    d["ri"] = np.ctypeslib.as_array(h.ri)[:n].copy()
    return d


def renorm_float(c):
    """The value a coefficient takes through copyspecout and copyspecin
    (divided by sqrt(2 pi), rounded to float, multiplied back)."""
    import sigio_oracle as so

    S = so.RENORM
    f = lambda x: (np.asarray(x) / S).astype(np.float32).astype(np.float64) * S
    c = np.asarray(c)
    return f(c.real) + 1j * f(c.imag)
