"""CPU model of the device apply over a ragged build (test helper).

Executes the same five phases as skelfmm_gb300/csrc/skf_apply.cu with numpy,
so the ragged layout produced on the host can be checked without a GPU.
"""
import numpy as np

from oracle import skel_oracle as O

_OPS = ["laplace_2d", "laplace_3d", "helmholtz_2d", "helmholtz_3d", "laplace_double_layer_3d",
        "laplace_adjoint_double_layer_3d", "helmholtz_double_layer_3d", "helmholtz_adjoint_double_layer_3d"]


def ragged_apply(rb, x):
    op = O.OPERATORS[_OPS[rb.op]]
    dt = np.complex128 if op.is_complex else np.float64
    E = rb.nentries
    q = np.zeros(E, dt)
    qh = np.zeros(E, dt)
    q[rb.perm_entry] = x[rb.perm_point]
    off, rk = rb.box_off, rb.box_rank
    lev = rb.box_level

    def T(b):
        r, s = int(rk[b]), int(off[b + 1] - off[b])
        return rb.t_data[rb.t_off[b]: rb.t_off[b] + r * (s - r)].reshape(r, s - r)

    for L in range(rb.nlevels - 1, rb.root_level, -1):
        for b in np.flatnonzero((lev == L) & (rk > 0)):
            o, r = off[b], int(rk[b])
            s = int(off[b + 1] - o)
            v = q[o: o + r] + T(b) @ q[o + r: o + s]
            qh[o: o + r] = v
            ps = rb.entry_pslot[o: o + r]
            q[ps[ps >= 0]] = v[ps >= 0]
    u = np.zeros(E, dt)
    uh = np.zeros(E, dt)
    for U in range(rb.nboxes):
        oU, rU = off[U], int(rk[U])
        XU = rb.entry_xyz[oU: off[U + 1]]
        GU = None if rb.entry_geom is None else rb.entry_geom[oU: off[U + 1]]
        for l in range(rb.list_off[U], rb.list_off[U + 1]):
            s, kind = int(rb.list_src[l]), int(rb.list_kind[l])
            oS, rS = off[s], int(rk[s])
            XS = rb.entry_xyz[oS: off[s + 1]]
            GS = None if rb.entry_geom is None else rb.entry_geom[oS: off[s + 1]]
            K = op.matrix(XU, XS, geom_trg=GU, geom_src=GS, param=rb.kappa)
            qs, qhs = q[oS: off[s + 1]], qh[oS: off[s + 1]]
            u[oU: off[U + 1]] += K @ qs
            if kind == 0:
                uh[oU: oU + rU] -= K[:rU, :rS] @ qhs[:rS]
            elif kind == 1:
                uh[oU: oU + rU] -= K[:rU] @ qs
            elif kind == 2:
                u[oU: off[U + 1]] -= K[:, :rS] @ qhs[:rS]
    for L in range(rb.root_level + 1, rb.nlevels):
        for b in np.flatnonzero((lev == L) & (rk > 0)):
            o, r = off[b], int(rk[b])
            s = int(off[b + 1] - o)
            ps = rb.entry_pslot[o: o + r]
            h = uh[o: o + r].copy()
            h[ps >= 0] += u[ps[ps >= 0]]
            u[o: o + r] += h
            u[o + r: o + s] += T(b).T @ h
    y = np.zeros(rb.npoints, dt)
    y[rb.perm_point] = u[rb.perm_entry]
    return y
