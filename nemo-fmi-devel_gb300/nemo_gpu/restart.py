"""Restart snapshots of a context's device state.

The variable set is that of the reference's ocean restart (rst_write,
restart.F90:133-191: rdt, kt, the before and now ub, vb, tb, sb, sshb, un, vn, tn,
sn, sshn, the masks and e3t_n/e3u_n/e3v_n) plus the barotropic extras of ts_rst
(dynspg_ts.F90:1440-1455: ub2_b, vb2_b, un_bf, vn_bf), under the reference's
variable names. NetCDF is not available here, so the file is a numpy .npz of
Fortran-order arrays: (jpi,jpj[,jpk]) for one member, with a leading member axis
for an ensemble. rhop (from eos, not on the path) is not written.

The device fields are copied through nemo_gpu_field_download / _upload (the C ABI)
in the precision they are held in, so a write followed by a read restores the
state bit for bit and the run continues as if uninterrupted. The now and before
barotropic velocities un_b, vn_b, ub_b, vb_b, which the reference recomputes from
un and ub when it reads a restart, are written as well; when a file lacks them
(a restart of the reference itself) they are recomputed here from un, vn, ub, vb
and the rest-state depths (linear free surface).
"""
import numpy as np

from . import api

# restart variable -> (field, tracer index or None)
STATE = {
    "ub": ("UB", None), "vb": ("VB", None), "tb": ("TSB", 0), "sb": ("TSB", 1), "sshb": ("SSHB", None),
    "un": ("UN", None), "vn": ("VN", None), "tn": ("TSN", 0), "sn": ("TSN", 1), "sshn": ("SSHN", None),
    "ub2_b": ("UB2_B", None), "vb2_b": ("VB2_B", None), "un_bf": ("UN_BF", None), "vn_bf": ("VN_BF", None),
    "un_b": ("UN_B", None), "vn_b": ("VN_B", None), "ub_b": ("UB_B", None), "vb_b": ("VB_B", None),
}
_3D = ("UB", "VB", "UN", "VN")
_TS = ("TSB", "TSN")


def _shape(ctx, field):
    jpi, jpj, jpk = ctx.jpi, ctx.jpj, ctx.jpk
    if field in _TS:
        return (jpi, jpj, jpk, 2)
    if field in _3D:
        return (jpi, jpj, jpk)
    return (jpi, jpj)


def _host(ctx, field):
    import torch
    n = ctx.field_numel(field) * ctx.nmem
    return torch.empty(n, dtype=ctx.field_dtype(field), pin_memory=True)


def _members(flat, shape, nmem):
    """(nmem, *shape) Fortran-order views of a flat member-outermost buffer."""
    a = flat.numpy()
    n = int(np.prod(shape))
    return [a[m * n:(m + 1) * n].reshape(shape, order="F") for m in range(nmem)]


def rst_write(ctx, path, kt):
    """Write the restart variables of the bound fields of ctx (all members) to path."""
    out = {"rdt": np.float64(ctx.nam["rn_rdt"]), "kt": np.float64(kt)}
    host = {}
    for field in {f for f, _ in STATE.values()}:
        if field not in ctx.bound:
            raise api.NemoError(f"rst_write: field {field} is not bound")
        host[field] = _host(ctx, field)
        ctx.download(field, host[field])
    ctx.synchronize()
    for name, (field, n) in STATE.items():
        arrs = _members(host[field], _shape(ctx, field), ctx.nmem)
        if n is not None:
            arrs = [a[..., n] for a in arrs]
        out[name] = np.asfortranarray(arrs[0]) if ctx.nmem == 1 else np.stack(arrs)
    from . import gyre
    tm, um, vm, _ = gyre.masks(ctx.dom)
    out.update(tmask=tm, umask=um, vmask=vm, smask=tm.max(axis=2))
    e3 = ctx.dom
    out.update(e3t_n=e3["e3t_0"], e3u_n=e3["e3u_0"], e3v_n=e3["e3v_0"])
    np.savez(path, **out)


def rst_read(ctx, path):
    """Upload the restart variables of path into the bound fields of ctx; returns the
    time step kt the restart was written at."""
    with np.load(path) as z:
        v = {k: z[k] for k in z.files}
    if abs(float(v["rdt"]) - ctx.nam["rn_rdt"]) > 0:
        raise api.NemoError("rst_read: the restart's rdt differs from the namelist's")
    if "un_b" not in v:
        _barotropic(ctx, v)
    fields = {}
    for name, (field, n) in STATE.items():
        a = v[name]
        arrs = [a] if ctx.nmem == 1 else list(a)
        fields.setdefault(field, [None] * ctx.nmem)
        for m, x in enumerate(arrs):
            if n is None:
                fields[field][m] = x
            else:
                if fields[field][m] is None:
                    fields[field][m] = np.zeros(_shape(ctx, field), order="F")
                fields[field][m][..., n] = x
    host = {}
    for field, arrs in fields.items():
        h = _host(ctx, field)
        h.numpy()[...] = np.concatenate([np.asarray(x).ravel(order="F") for x in arrs]).astype(h.numpy().dtype)
        host[field] = h
        ctx.upload(field, h)
    ctx.synchronize()
    return int(v["kt"])


def _barotropic(ctx, v):
    """un_b, ub_b, vn_b, vb_b from the 3-D velocities (dynnxt.F90:345-358, rest-state
    depths) for a restart written without them."""
    from . import gyre
    _, um, vm, _ = gyre.masks(ctx.dom)
    d = ctx.dom
    hu = (d["e3u_0"] * um)[:, :, :-1].sum(axis=2)
    hv = (d["e3v_0"] * vm)[:, :, :-1].sum(axis=2)
    r1u = np.where(hu > 0, 1.0 / np.where(hu > 0, hu, 1.0), 0.0)
    r1v = np.where(hv > 0, 1.0 / np.where(hv > 0, hv, 1.0), 0.0)
    for bt, fld, e3, msk, r1 in (("un_b", "un", "e3u_0", um, r1u), ("ub_b", "ub", "e3u_0", um, r1u),
                                 ("vn_b", "vn", "e3v_0", vm, r1v), ("vb_b", "vb", "e3v_0", vm, r1v)):
        s = ((d[e3] * msk)[..., :-1] * v[fld][..., :-1]).sum(axis=-1)   # levels 1..jpk-1
        v[bt] = s * r1
