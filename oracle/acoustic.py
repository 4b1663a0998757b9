"""CPU restatement of the reference's 2-D acoustic staggered-grid loop (test oracle).

Follows ``ADFWI/propagator/acoustic_kernels.py`` of the reference:

* ``pad_edge``            <- ``pad_torchSingle`` (lines 16-37): edge-replicate pad;
* ``acoustic_forward_coef`` <- ``forward_kernel`` lines 252-265 (kappa1, kappa2, kappa3,
  c1 = 9/8, c2 = -1/24) and the loop of lines 239-301 given alpha1, alpha2;
* ``_step``               <- ``step_forward`` lines 113-174 (p update, source,
  free-surface mirror, u and w updates, w mirror, receiver gather,
  illumination sums);
* ``acoustic_forward``    <- ``forward_kernel`` lines 224-301 (padding,
  index shift by nabc, zero fields, chunked time loop, record dict, and the
  forward_wavefield_u / _w accumulation order of lines 172-174 and 285-288).

Test infrastructure only: never imported by the product package.
"""
import torch
import torch.utils.checkpoint

C1 = 9.0 / 8.0
C2 = -1.0 / 24.0


def _cpu_only(*ts, allow_gpu=False):
    """The oracle checks results on the CPU. ``allow_gpu`` lets a timing test run the same
    PyTorch loop on CUDA tensors as the plain (reference-shaped) GPU path it is compared to."""
    if allow_gpu:
        return
    for t in ts:
        if torch.is_tensor(t) and t.device.type != "cpu":
            raise RuntimeError("oracle runs on the CPU only")


def pad_edge(v, nabc):
    """Edge-replicate padding by ``nabc`` cells on all four sides (acoustic_kernels.py:16-37)."""
    return torch.nn.functional.pad(v[None, None], (nabc, nabc, nabc, nabc), mode="replicate")[0, 0]


def _step(p, u, w, it, co, src, rcv, fs, free_surface, dt, nabc, nz, nx):
    """One time step (acoustic_kernels.py:113-174). Returns new fields, records, squares."""
    alpha1, kappa1, alpha2, kappa2, kappa3 = co
    sz, sx, wav = src
    rz, rx = rcv
    ns, nzp, nxp = p.shape
    zi = slice(fs + 1, nzp - 2)
    xi = slice(2, nxp - 2)
    pn = p.clone()
    pn[:, zi, xi] = ((1.0 - kappa1[zi, xi]) * p[:, zi, xi] - alpha1[zi, xi] * (
        C1 * (u[:, zi, 2:nxp - 2] - u[:, zi, 1:nxp - 3]
              + w[:, fs + 1:nzp - 2, xi] - w[:, fs:nzp - 3, xi])
        + C2 * (u[:, zi, 3:nxp - 1] - u[:, zi, 0:nxp - 4]
                + w[:, fs + 2:nzp - 1, xi] - w[:, fs - 1:nzp - 4, xi])))
    shots = torch.arange(ns, device=p.device)
    pn[shots, sz, sx] = pn[shots, sz, sx] + dt * wav[:, it]
    if free_surface:
        pn[:, fs - 1, :] = -pn[:, fs + 1, :]
    un = u.clone()
    zu = slice(fs, nzp - 1)
    xu = slice(1, nxp - 2)
    un[:, zu, xu] = ((1.0 - kappa2[zu, xu]) * u[:, zu, xu] - alpha2[zu, xu] * (
        C1 * (pn[:, zu, 2:nxp - 1] - pn[:, zu, 1:nxp - 2])
        + C2 * (pn[:, zu, 3:nxp] - pn[:, zu, 0:nxp - 3])))
    wn = w.clone()
    zw = slice(fs, nzp - 2)
    xw = slice(1, nxp - 1)
    wn[:, zw, xw] = ((1.0 - kappa3[zw, xw]) * w[:, zw, xw] - alpha2[zw, xw] * (
        C1 * (pn[:, fs + 1:nzp - 1, xw] - pn[:, fs:nzp - 2, xw])
        + C2 * (pn[:, fs + 2:nzp, xw] - pn[:, fs - 1:nzp - 3, xw])))
    if free_surface:
        wn[:, fs - 1, :] = wn[:, fs, :]
    rec = (pn[:, rz, rx], un[:, rz, rx], wn[:, rz, rx])
    inner = (slice(nabc, nabc + nz), slice(nabc, nabc + nx))
    sq = (torch.sum(pn * pn, dim=0)[inner].detach(),
          torch.sum(un * un, dim=0)[inner].detach(),
          torch.sum(wn * wn, dim=0)[inner].detach())
    return pn, un, wn, rec, sq


def acoustic_forward(vp, rho, damp, src_x, src_z, wavelet, rcv_x, rcv_z, *, nabc, free_surface,
                     dx, dz, dt, checkpoint_segments=1, allow_gpu=False, checkpoint_chunks=False):
    """Records of the reference acoustic propagator (acoustic_kernels.py:179-301).

    ``vp``, ``rho``: (nz, nx); ``damp``: (nz+2nabc, nx+2nabc); ``src_*``: int (ns,);
    ``wavelet``: (ns, nt); ``rcv_*``: int (nr,). Returns the reference's record dict.
    Differentiable w.r.t. ``vp`` and ``rho`` through autograd.
    """
    _cpu_only(vp, rho, damp, wavelet, allow_gpu=allow_gpu)
    c = pad_edge(vp, nabc)
    den = pad_edge(rho, nabc)
    alpha1 = den * c * c * dt / dz
    alpha2 = dt / (den * dz)
    return acoustic_forward_coef(alpha1, alpha2, damp, src_x, src_z, wavelet, rcv_x, rcv_z, nabc=nabc,
                                 free_surface=free_surface, dt=dt, checkpoint_segments=checkpoint_segments,
                                 allow_gpu=allow_gpu, checkpoint_chunks=checkpoint_chunks)


def acoustic_forward_coef(alpha1, alpha2, damp, src_x, src_z, wavelet, rcv_x, rcv_z, *, nabc, free_surface, dt,
                          checkpoint_segments=1, allow_gpu=False, checkpoint_chunks=False):
    """The time loop of acoustic_kernels.py:239-301 given alpha1 = rho c^2 dt/dz and
    alpha2 = dt/(rho dz) on the padded grid (differentiable w.r.t. both). ``checkpoint_chunks``
    runs every chunk under torch.utils.checkpoint as the reference does (same values; the
    backward recomputes the chunk), for timing the reference's memory-bounded mode."""
    _cpu_only(alpha1, alpha2, damp, wavelet, allow_gpu=allow_gpu)
    nzp, nxp = alpha1.shape
    nz, nx = nzp - 2 * nabc, nxp - 2 * nabc
    dtype = alpha1.dtype
    dev = alpha1.device
    fs = nabc if free_surface else 1
    sx = torch.as_tensor(src_x, dtype=torch.long, device=dev) + nabc
    sz = torch.as_tensor(src_z, dtype=torch.long, device=dev) + nabc
    rx = torch.as_tensor(rcv_x, dtype=torch.long, device=dev) + nabc
    rz = torch.as_tensor(rcv_z, dtype=torch.long, device=dev) + nabc
    ns = sx.numel()
    damp = damp.to(dtype)
    kappa1 = damp * dt
    kappa2 = torch.zeros_like(damp)
    kappa2[:, 1:nxp - 2] = 0.5 * (damp[:, 1:nxp - 2] + damp[:, 2:nxp - 1]) * dt
    kappa3 = torch.zeros_like(damp)
    kappa3[fs:nzp - 2, :] = 0.5 * (damp[fs:nzp - 2, :] + damp[fs + 1:nzp - 1, :]) * dt
    co = (alpha1, kappa1, alpha2, kappa2, kappa3)
    p = torch.zeros((ns, nzp, nxp), dtype=dtype, device=dev)
    u = torch.zeros((ns, nzp, nxp - 1), dtype=dtype, device=dev)
    w = torch.zeros((ns, nzp - 1, nxp), dtype=dtype, device=dev)
    fwp = torch.zeros((nz, nx), dtype=dtype, device=dev)
    fwu = torch.zeros((nz, nx), dtype=dtype, device=dev)
    fww = torch.zeros((nz, nx), dtype=dtype, device=dev)
    def run_chunk(p, u, w, chunk, alpha1, alpha2):
        cc = (alpha1, kappa1, alpha2, kappa2, kappa3)
        rec_chunk = ([], [], [])
        seg_p = torch.zeros((nz, nx), dtype=dtype, device=dev)
        seg_u = torch.zeros((nz, nx), dtype=dtype, device=dev)
        seg_w = torch.zeros((nz, nx), dtype=dtype, device=dev)
        for it in range(chunk.shape[-1]):
            p, u, w, rec, sq = _step(p, u, w, it, cc, (sz, sx, chunk), (rz, rx), fs, free_surface,
                                     dt, nabc, nz, nx)
            for lst, r in zip(rec_chunk, rec):
                lst.append(r)
            seg_p = seg_p + sq[0]
            seg_u = seg_u + sq[1]
            seg_w = seg_u + sq[2]
        return (p, u, w) + tuple(torch.stack(lst, dim=1) for lst in rec_chunk) + (seg_p, seg_u, seg_w)

    recs = ([], [], [])
    for chunk in torch.chunk(wavelet, checkpoint_segments, dim=-1):
        if checkpoint_chunks:
            # the reference runs each chunk under torch.utils.checkpoint (acoustic_kernels.py:268-278)
            res = torch.utils.checkpoint.checkpoint(run_chunk, p, u, w, chunk, alpha1, alpha2, use_reentrant=True)
        else:
            res = run_chunk(p, u, w, chunk, alpha1, alpha2)
        p, u, w = res[:3]
        for lst, r in zip(recs, res[3:6]):
            lst.append(r)
        seg_p, seg_u, seg_w = res[6:]
        fwp = fwp + seg_p
        fwu = fwp + seg_u
        fww = fwp + seg_w
    out = {}
    for key, lst in zip(("p", "u", "w"), recs):
        out[key] = torch.cat(lst, dim=1)
    out["forward_wavefield_p"] = fwp
    out["forward_wavefield_u"] = fwu
    out["forward_wavefield_w"] = fww
    return out
