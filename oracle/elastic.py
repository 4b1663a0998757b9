"""CPU restatement of the reference's 2-D velocity-stress elastic loop (test oracle).

Follows ``ADFWI/propagator/elastic_kernels.py`` of the reference:

* ``diff_coef``        <- ``DiffCoef`` (lines 20-58, grid scheme 's');
* ``_dxf/_dxb/_dzf/_dzb`` <- ``Dxfm_4 .. Dzbm_6`` (lines 66-108): staggered
  half-cell derivatives on the index ranges ii = [NN, nzp-NN), jj = [NN, nxp-NN);
* ``pad_elastic``      <- ``pad_torchSingle`` (lines 175-216);
* ``_step_pml``        <- ``step_forward_PML_4order/_6order`` loop bodies
  (lines 339-418 and 495-574): split-field PML, moment-tensor source
  (-MT/2 on both split parts), totals, free-surface rows h-3..h-1,
  5-component receivers, per-step (not accumulated) energy;
* ``_step_abl``        <- ``step_forward_ABL_4order/_6order`` loop bodies
  (lines 709-774 and 844-909): unsplit update, -MT/3 source, multiplicative
  damping of the velocities;
* ``elastic_forward``  <- ``forward_kernel`` (lines 917-1037).

Test infrastructure only: never imported by the product package.
"""
import torch

from .acoustic import _cpu_only


def diff_coef(nn):
    """Staggered-grid coefficients from a float32 linear solve (elastic_kernels.py:20-58)."""
    a = torch.empty((nn, nn), dtype=torch.float32)
    for i in range(nn):
        for j in range(nn):
            a[i, j] = (2 * (j + 1) - 1) ** (2 * (i + 1) - 1)
    b = torch.cat((torch.tensor([1.0], dtype=torch.float32), torch.zeros(nn - 1, dtype=torch.float32)))
    return torch.linalg.inv(a) @ b


def _dxf(a, f, nn):
    """Forward x difference on [NN, n-NN): sum_k f_k (a[j+1+k] - a[j-k]) (Dxfm_*)."""
    n = a.shape[-1]
    out = None
    for k in range(len(f)):
        term = f[k] * (a[:, nn:a.shape[1] - nn, nn + 1 + k:n - nn + 1 + k]
                       - a[:, nn:a.shape[1] - nn, nn - k:n - nn - k])
        out = term if out is None else out + term
    return out


def _dxb(a, f, nn):
    """Backward x difference: sum_k f_k (a[j+k] - a[j-1-k]) (Dxbm_*)."""
    n = a.shape[-1]
    out = None
    for k in range(len(f)):
        term = f[k] * (a[:, nn:a.shape[1] - nn, nn + k:n - nn + k]
                       - a[:, nn:a.shape[1] - nn, nn - 1 - k:n - nn - 1 - k])
        out = term if out is None else out + term
    return out


def _dzf(a, f, nn):
    """Forward z difference (Dzfm_*)."""
    m = a.shape[1]
    out = None
    for k in range(len(f)):
        term = f[k] * (a[:, nn + 1 + k:m - nn + 1 + k, nn:a.shape[2] - nn]
                       - a[:, nn - k:m - nn - k, nn:a.shape[2] - nn])
        out = term if out is None else out + term
    return out


def _dzb(a, f, nn):
    """Backward z difference (Dzbm_*)."""
    m = a.shape[1]
    out = None
    for k in range(len(f)):
        term = f[k] * (a[:, nn + k:m - nn + k, nn:a.shape[2] - nn]
                       - a[:, nn - 1 - k:m - nn - 1 - k, nn:a.shape[2] - nn])
        out = term if out is None else out + term
    return out


def pad_elastic(data, pml, fs_offset, free_surface):
    """Edge-replicate pad, top = fs_offset (+pml without free surface) (elastic_kernels.py:175-216)."""
    top = fs_offset if free_surface else fs_offset + pml
    return torch.nn.functional.pad(data[None, None], (pml, pml, top, pml), mode="replicate")[0, 0]


def _apply_fs_stress(tzz, txz, h):
    tzz = tzz.clone()
    txz = txz.clone()
    tzz[:, h - 1, :] = 0
    tzz[:, h - 2, :] = -tzz[:, h, :]
    txz[:, h - 2, :] = -txz[:, h - 1, :]
    txz[:, h - 3, :] = -txz[:, h, :]
    return tzz, txz


def _apply_fs_velocity(vx, vz, h, js, je):
    vx = vx.clone()
    vz = vz.clone()
    jj = slice(js, je + 1)
    jp = slice(js + 1, je + 2)
    vz[:, h - 2, jj] = vz[:, h - 1, jj]
    vx[:, h - 2, jj] = vz[:, h - 2, jp] - vz[:, h - 2, jj] + vz[:, h - 1, jp] - vz[:, h - 1, jj] + vx[:, h, jj]
    vz[:, h - 3, jj] = vz[:, h - 2, jj]
    return vx, vz


def _set(a, region, val):
    a = a.clone()
    a[(slice(None),) + region] = val
    return a


def _add_src(a, shots, sz, sx, val):
    a = a.clone()
    a[shots, sz, sx] = a[shots, sz, sx] + val
    return a


def elastic_forward(coef, src_x, src_z, wavelet, mt, rcv_x, rcv_z, *, nabc, free_surface, dx, dz, dt,
                    fd_order=4, abc_type="PML", bcx=None, bcz=None, damp=None, checkpoint_segments=1):
    """Records of the reference elastic propagator (elastic_kernels.py:917-1037).

    ``coef`` maps C11, C13, C15, C33, C35, C55, bx, bz to the UNPADDED model-side tensors
    (C55: (nz-2, nx-2), bx: (nz, nx-1), bz: (nz-1, nx)). ``bcx``/``bcz`` (PML) or ``damp``
    (other abc types) come unpadded as the boundary functions return them.
    Differentiable w.r.t. every tensor in ``coef``.
    """
    if fd_order not in (4, 6):
        raise ValueError("fd_order must be 4 or 6")
    _cpu_only(wavelet, *coef.values())
    nz, nx = coef["C11"].shape
    dtype = coef["C11"].dtype
    fs_off = fd_order // 2
    nn = fd_order // 2
    h = nn + 1
    nxp = nx + 2 * nabc
    nzp = nz + (nabc + fs_off if free_surface else 2 * nabc + fs_off)
    pad = {k: pad_elastic(v, nabc, fs_off, free_surface) for k, v in coef.items()}
    pml = abc_type.lower() == "pml"
    if pml:
        bcx = pad_elastic(torch.as_tensor(bcx, dtype=dtype), 0, fs_off, free_surface)
        bcz = pad_elastic(torch.as_tensor(bcz, dtype=dtype), 0, fs_off, free_surface)
    else:
        damp = pad_elastic(torch.as_tensor(damp, dtype=dtype), 0, fs_off, free_surface)
    sx = torch.as_tensor(src_x, dtype=torch.long) + nabc
    sz = torch.as_tensor(src_z, dtype=torch.long) + (fs_off if free_surface else nabc + fs_off)
    rx = torch.as_tensor(rcv_x, dtype=torch.long) + nabc
    rz = torch.as_tensor(rcv_z, dtype=torch.long) + (fs_off if free_surface else nabc + fs_off)
    ns = sx.numel()
    shots = torch.arange(ns)
    f = diff_coef(nn)
    fl = [f[k] for k in range(nn)]
    ie = nzp - nn - 1
    je = nxp - nn - 1
    reg = (slice(nn, ie + 1), slice(nn, je + 1))
    C = {k: v[reg] for k, v in pad.items()}
    mt = torch.as_tensor(mt, dtype=dtype)
    z = lambda: torch.zeros((ns, nzp, nxp), dtype=dtype)  # noqa: E731
    offset = fs_off if free_surface else fs_off + nabc
    inner = (slice(offset, offset + nz), slice(nabc, nabc + nx))
    names = ("txx", "tzz", "txz", "vx", "vz")
    recs = {k: [] for k in names}
    fw = {k: torch.zeros((nz, nx), dtype=dtype) for k in names}
    if pml:
        pmlxd = 1 + 0.5 * dt * bcx[reg]
        pmlxn = 1 - 0.5 * dt * bcx[reg]
        pmlzd = 1 + 0.5 * dt * bcz[reg]
        pmlzn = 1 - 0.5 * dt * bcz[reg]
        dt_dx = dt / dx
        dt_dz = dt / dz
        pmlx_inv = 1.0 / pmlxd
        pmlz_inv = 1.0 / pmlzd
        half_mt = mt / 2
        st = {k: z() for k in ("txx_x", "txx_z", "tzz_x", "tzz_z", "txz_x", "txz_z",
                               "vx_x", "vx_z", "vz_x", "vz_z", "txx", "tzz", "txz", "vx", "vz")}
    else:
        st = {k: z() for k in names}
    for chunk in torch.chunk(wavelet, checkpoint_segments, dim=-1):
        last = None
        for t in range(chunk.shape[-1]):
            vx, vz = st["vx"], st["vz"]
            dxbm_vx = _dxb(vx, fl, nn)
            dxbm_vz = _dxb(vz, fl, nn)
            dzbm_vx = _dzb(vx, fl, nn)
            dzbm_vz = _dzb(vz, fl, nn)
            dxfm_vx = _dxf(vx, fl, nn)
            dzfm_vx = _dzf(vx, fl, nn)
            dxfm_vz = _dxf(vz, fl, nn)
            dzfm_vz = _dzf(vz, fl, nn)
            if pml:
                s = st
                s["txx_x"] = _set(s["txx_x"], reg, (pmlxn * s["txx_x"][(slice(None),) + reg] + dt_dx * (C["C11"] * dxbm_vx + C["C15"] * dxbm_vz)) * pmlx_inv)
                s["txx_z"] = _set(s["txx_z"], reg, (pmlzn * s["txx_z"][(slice(None),) + reg] + dt_dz * (C["C15"] * dzbm_vx + C["C13"] * dzbm_vz)) * pmlz_inv)
                s["tzz_x"] = _set(s["tzz_x"], reg, (pmlxn * s["tzz_x"][(slice(None),) + reg] + dt_dx * (C["C13"] * dxbm_vx + C["C35"] * dxbm_vz)) * pmlx_inv)
                s["tzz_z"] = _set(s["tzz_z"], reg, (pmlzn * s["tzz_z"][(slice(None),) + reg] + dt_dz * (C["C35"] * dzbm_vx + C["C33"] * dzbm_vz)) * pmlz_inv)
                s["txz_x"] = _set(s["txz_x"], reg, (pmlxn * s["txz_x"][(slice(None),) + reg] + dt_dx * (C["C15"] * dxfm_vx + C["C55"] * dxfm_vz)) * pmlx_inv)
                s["txz_z"] = _set(s["txz_z"], reg, (pmlzn * s["txz_z"][(slice(None),) + reg] + dt_dz * (C["C55"] * dzfm_vx + C["C35"] * dzfm_vz)) * pmlz_inv)
                w = chunk[:, t]
                for part in ("_x", "_z"):
                    s["txx" + part] = _add_src(s["txx" + part], shots, sz, sx, -half_mt[:, 0, 0] * w)
                    s["tzz" + part] = _add_src(s["tzz" + part], shots, sz, sx, -half_mt[:, 2, 2] * w)
                    s["txz" + part] = _add_src(s["txz" + part], shots, sz, sx, -half_mt[:, 0, 2] * w)
                txx = s["txx_x"] + s["txx_z"]
                tzz = s["tzz_x"] + s["tzz_z"]
                txz = s["txz_x"] + s["txz_z"]
                if free_surface:
                    tzz, txz = _apply_fs_stress(tzz, txz, h)
                dxfm_txx = _dxf(txx, fl, nn)
                dzbm_txz = _dzb(txz, fl, nn)
                dxbm_txz = _dxb(txz, fl, nn)
                dzfm_tzz = _dzf(tzz, fl, nn)
                s["vx_x"] = _set(s["vx_x"], reg, (pmlxn * s["vx_x"][(slice(None),) + reg] + dt * C["bx"] * dxfm_txx / dx) / pmlxd)
                s["vx_z"] = _set(s["vx_z"], reg, (pmlzn * s["vx_z"][(slice(None),) + reg] + dt * C["bx"] * dzbm_txz / dz) / pmlzd)
                s["vz_x"] = _set(s["vz_x"], reg, (pmlxn * s["vz_x"][(slice(None),) + reg] + dt * C["bz"] * dxbm_txz / dx) / pmlxd)
                s["vz_z"] = _set(s["vz_z"], reg, (pmlzn * s["vz_z"][(slice(None),) + reg] + dt * C["bz"] * dzfm_tzz / dz) / pmlzd)
                vx = s["vx_x"] + s["vx_z"]
                vz = s["vz_x"] + s["vz_z"]
                if free_surface:
                    vx, vz = _apply_fs_velocity(vx, vz, h, nn, je)
                s["txx"], s["tzz"], s["txz"], s["vx"], s["vz"] = txx, tzz, txz, vx, vz
            else:
                s = st
                R = (slice(None),) + reg
                txx = _set(s["txx"], reg, s["txx"][R] + dt * ((C["C11"] * dxbm_vx + C["C15"] * dxbm_vz) / dx
                                                          + (C["C15"] * dzbm_vx + C["C13"] * dzbm_vz) / dz))
                tzz = _set(s["tzz"], reg, s["tzz"][R] + dt * ((C["C13"] * dxbm_vx + C["C35"] * dxbm_vz) / dx
                                                          + (C["C35"] * dzbm_vx + C["C33"] * dzbm_vz) / dz))
                txz = _set(s["txz"], reg, s["txz"][R] + dt * ((C["C15"] * dxfm_vx + C["C55"] * dxfm_vz) / dx
                                                          + (C["C55"] * dzfm_vx + C["C35"] * dzfm_vz) / dz))
                w = chunk[:, t]
                sc = -1 / 3
                txx = _add_src(txx, shots, sz, sx, sc * mt[:, 0, 0] * w)
                tzz = _add_src(tzz, shots, sz, sx, sc * mt[:, 2, 2] * w)
                txz = _add_src(txz, shots, sz, sx, sc * mt[:, 0, 2] * w)
                if free_surface:
                    tzz, txz = _apply_fs_stress(tzz, txz, h)
                dxfm_txx = _dxf(txx, fl, nn)
                dzbm_txz = _dzb(txz, fl, nn)
                dxbm_txz = _dxb(txz, fl, nn)
                dzfm_tzz = _dzf(tzz, fl, nn)
                vx = _set(s["vx"], reg, s["vx"][R] + dt * C["bx"] * (dxfm_txx / dx + dzbm_txz / dz))
                vz = _set(s["vz"], reg, s["vz"][R] + dt * C["bz"] * (dxbm_txz / dx + dzfm_tzz / dz))
                if free_surface:
                    vx, vz = _apply_fs_velocity(vx, vz, h, nn, je)
                vx = vx * damp
                vz = vz * damp
                s["txx"], s["tzz"], s["txz"], s["vx"], s["vz"] = txx, tzz, txz, vx, vz
            for k in names:
                recs[k].append(s[k][:, rz, rx])
            last = {k: torch.sum(s[k] * s[k], dim=0)[inner].detach() for k in names}
        for k in names:
            fw[k] = fw[k] + last[k]
    out = {k: torch.stack(recs[k], dim=1) for k in names}
    for k in names:
        out["forward_wavefield_" + k] = fw[k]
    return out
