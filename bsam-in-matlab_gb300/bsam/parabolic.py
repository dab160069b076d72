"""Parabolic driver (host), mirroring ``ParabolicBSAM/src``.

    du/dt - div(D grad u) + C u = f

Implicit BE / BDF2 / CN stepping: every step is one mass-conservative AFAS
solve with C_eff = C + alpha/Dt (``ebpSolve.m:37-78``), and the hierarchy
follows the solution by periodic conservative regridding
(``ebpRegrid.m:16-162``).  Right-hand sides, coefficient refreshes and the
regrid transfer are host set-up work, as in the reference; every
``ebSolveCycles``, ghost fill, prolongation and fill-down runs through the
backend (the CUDA library in the product).
"""
from __future__ import annotations

import math

import numpy as np

from . import hierarchy as hier
from .options import Options, ebOptions
from .problem import ebProblem, Problem, SIDES
from .solve import ebSolveCycles, default_backend, error_norms
from .tagcluster import tag_cluster, _nargin


def _wrapT(v, label):
    """(x,y) or (x,y,t) callables, or scalars -> (f(x,y,t), time-dependent)
    (``ebpProblem.m:59-79``)."""
    if callable(v):
        na = _nargin(v)
        if na == 3:
            return v, True
        if na == 2:
            return (lambda X, Y, T: v(X, Y)), False
        raise ValueError(f'ebp_problem:arity: {label} must take (x,y) or (x,y,t).')
    if np.isscalar(v) and np.isreal(v):
        vv = float(v)
        return (lambda X, Y, T: vv * np.ones(np.shape(X))), False
    raise ValueError(f'ebp_problem:badinput: {label} must be a handle or scalar.')


def ebpProblem(domain, D, C, f, bc, u0, exact=None) -> Problem:
    """``ebpProblem.m:1-56``."""
    domain = [float(v) for v in domain]
    if len(domain) != 4 or domain[1] <= domain[0] or domain[3] <= domain[2]:
        raise ValueError('ebp_problem:domain: domain must be [a b c d].')
    p = Problem()
    p.domain = domain
    p.D, p.tdD = _wrapT(D, 'D')
    p.C, p.tdC = _wrapT(C, 'C')
    p.f, p.tdF = _wrapT(f, 'f')
    p.fzero = np.isscalar(f) and float(f) == 0.0    # lets a device step skip sampling f
    if isinstance(bc, (list, tuple)) and len(bc) == 2 and isinstance(bc[0], str):
        bc = {s: bc for s in SIDES}
    p.tdBC = False
    p.bc = []
    for s in SIDES:
        t = str(bc[s][0]).lower()
        if t not in ('dirichlet', 'neumann'):
            raise ValueError('ebp_problem:bc: bc type must be dirichlet or neumann')
        g, td = _wrapT(bc[s][1], 'g_' + s)
        p.bc.append({'type': t, 'g': g})
        p.tdBC = p.tdBC or td
    if not callable(u0):
        raise ValueError('ebp_problem:u0: u0 must be @(X,Y).')
    p.u0 = u0
    p.exact = exact
    return p


_TIME = {'Scheme': 'bdf2', 'Dt': None, 'TFinal': None, 'RegridEvery': 8, 'StepVerbose': 10, 'Callback': None,
         'MaxVCyclesStep': 20}


def ebpOptions(*args, **kwargs) -> Options:
    """``ebpOptions.m:18-58``: time options; the rest go to ebOptions."""
    if len(args) % 2:
        raise ValueError('ebp_options:pairs: Options must be name-value pairs.')
    pairs = list(zip(args[0::2], args[1::2])) + list(kwargs.items())
    opts = Options(dict(_TIME))
    rest = []
    lower = {k.lower(): k for k in _TIME}
    for nm, v in pairs:
        k = lower.get(str(nm).lower())
        if k is not None:
            opts[k] = v
        else:
            rest += [nm, v]
    opts.Scheme = str(opts.Scheme).lower()
    if opts.Scheme not in ('be', 'bdf2', 'cn'):
        raise ValueError('ebp_options:scheme: Scheme must be be, bdf2 or cn.')
    if opts.Dt is None or opts.TFinal is None:
        raise ValueError('ebp_options:time: Dt and TFinal are required.')
    for nm in ('Dt', 'TFinal'):
        v = opts[nm]
        if not (np.isscalar(v) and np.isreal(v) and np.isfinite(v) and v > 0):
            raise ValueError(f'ebp_options:time: {nm} must be a positive finite real scalar.')
    for nm, lo in (('RegridEvery', 0), ('StepVerbose', 0), ('MaxVCyclesStep', 1)):
        v = opts[nm]
        if not (np.isscalar(v) and np.isreal(v) and np.isfinite(v) and float(v) == int(v) and v >= lo):
            raise ValueError(f'ebp_options:{nm.lower()}: {nm} must be an integer >= {lo}.')
    if opts.Callback is not None and not callable(opts.Callback):
        raise ValueError('ebp_options:callback: Callback must be empty or a function handle.')
    eb = ebOptions(*rest)
    eb.Verbose = 0
    eb.MaxVCycles = int(opts.MaxVCyclesStep)
    opts.eb = eb
    return opts


def ebpEprob(pprob, t, aDt):
    """Elliptic problem of one step (``ebpEprob.m``): C + alpha/Dt, f = 0."""
    bc = {}
    for s, side in enumerate(SIDES):
        g = pprob.bc[s]['g']
        bc[side] = (pprob.bc[s]['type'], (lambda gg: (lambda x, y: gg(x, y, t)))(g))
    return ebProblem(pprob.domain, lambda x, y: pprob.D(x, y, t), lambda x, y: pprob.C(x, y, t) + aDt,
                     lambda x, y: np.zeros(np.shape(x)), bc, None)


def _centres(H, k, p):
    lev = H.lev[k]
    b = lev.box[p]
    dom = H.prob.domain
    return np.meshgrid(dom[0] + (np.arange(b[0], b[1] + 1) - 0.5) * lev.h[0],
                       dom[2] + (np.arange(b[2], b[3] + 1) - 0.5) * lev.h[1], indexing='ij')


def _interiors(H):
    return {(k, p): H.lev[k].Q[p][1:-1, 1:-1].copy(order='F') for k in range(1, H.nlev + 1)
            for p in range(H.lev[k].np)}


def _set_u0(H, pprob, ks):
    for k in ks:
        for p in range(H.lev[k].np):
            X, Y = _centres(H, k, p)
            H.lev[k].Q[p][1:-1, 1:-1] = pprob.u0(X, Y)
    H.mark_dirty('Q')


def ebpInit(pprob, opts, aDt1, backend):
    """``ebpInit.m:9-30``: hierarchy adapted to u0."""
    H = hier.setup(ebpEprob(pprob, 0.0, aDt1), opts.eb, backend)
    _set_u0(H, pprob, range(1, H.nlev + 1))
    backend.run(H, [('fill', k) for k in range(1, H.nlev + 1)])
    while (H.nlev - H.rootIdx + 1) < opts.eb.MaxLevels:
        boxes = tag_cluster(H, backend)
        if boxes.shape[0] == 0:
            break
        H = hier.add_level(H, boxes, backend)
        _set_u0(H, pprob, [H.nlev])
        backend.run(H, [('fill', H.nlev)])
    backend.run(H, [('filldown',)])
    td = pprob.tdD or pprob.tdC or pprob.tdBC
    H.par = {'Uo': _interiors(H), 'Uoo': None, 'stateKey': (0.0 * td, aDt1), 'aDt': aDt1}
    return H


def _face_corrections(H, k, p):
    """``ebFaceCorrections.m:18-61`` on host arrays (CN right-hand side)."""
    lev = H.lev[k]
    Q, QC = lev.Q[p], lev.QC[p]
    DeW, DnS, cfD = lev.DeW[p], lev.DnS[p], lev.cfD[p]
    mx, my = Q.shape[0] - 2, Q.shape[1] - 2
    cmx, cmy = mx // 2, my // 2
    hcx2 = H.lev[k - 1].h[0] ** 2
    hcy2 = H.lev[k - 1].h[1] ** 2
    j = np.arange(1, cmy + 1)
    i = np.arange(1, cmx + 1)
    W = ((DeW[0, 2 * j - 2] * (Q[1, 2 * j - 1] - Q[0, 2 * j - 1]) + DeW[0, 2 * j - 1] * (Q[1, 2 * j] - Q[0, 2 * j]))
         + cfD['W'] * (QC[0, j] - QC[1, j])) / hcx2
    E = ((DeW[mx, 2 * j - 2] * (Q[mx, 2 * j - 1] - Q[mx + 1, 2 * j - 1])
          + DeW[mx, 2 * j - 1] * (Q[mx, 2 * j] - Q[mx + 1, 2 * j]))
         + cfD['E'] * (QC[cmx + 1, j] - QC[cmx, j])) / hcx2
    S = ((DnS[2 * i - 2, 0] * (Q[2 * i - 1, 1] - Q[2 * i - 1, 0]) + DnS[2 * i - 1, 0] * (Q[2 * i, 1] - Q[2 * i, 0]))
         + cfD['S'] * (QC[i, 0] - QC[i, 1])) / hcy2
    N = ((DnS[2 * i - 2, my] * (Q[2 * i - 1, my] - Q[2 * i - 1, my + 1])
          + DnS[2 * i - 1, my] * (Q[2 * i, my] - Q[2 * i, my + 1]))
         + cfD['N'] * (QC[i, cmy + 1] - QC[i, cmy])) / hcy2
    ops = lev.ops[p]
    return [(ops['corrW'], W), (ops['corrE'], E), (ops['corrS'], S), (ops['corrN'], N)]


def ebpRhs(H, pprob, t1, Dt, scheme, backend):
    """``ebpRhs.m:25-67``: FTrue of the step on every level >= root."""
    if scheme == 'cn':
        backend.run(H, [('filldown',)] + [('fill', k) for k in range(1, H.nlev + 1)])
    Uo = H.par['Uo']
    for k in range(H.rootIdx, H.nlev + 1):
        lev = H.lev[k]
        for p in range(lev.np):
            X, Y = _centres(H, k, p)
            uo = Uo[(k, p)]
            if scheme == 'be':
                FT = pprob.f(X, Y, t1) + uo / Dt
            elif scheme == 'bdf2':
                FT = pprob.f(X, Y, t1) + (2 * uo - 0.5 * H.par['Uoo'][(k, p)]) / Dt
            elif scheme == 'cn':
                Le = hier.op2d(lev.Q[p], lev.DeW[p], lev.DnS[p], lev.CC[p], lev.h[0], lev.h[1])
                FT = (2 * pprob.f(X, Y, t1 - Dt / 2) + (2 / Dt + H.par['aDt']) * uo) - Le
            else:
                raise ValueError(f'ebp_rhs:scheme: unknown scheme {scheme}')
            lev.FTrue[p] = np.asfortranarray(np.broadcast_to(FT, X.shape), dtype=np.float64)
    if scheme == 'cn' and H.opts.MassCorrection:
        for k in range(H.rootIdx + 1, H.nlev + 1):
            lev = H.lev[k]
            for p in range(lev.np):        # ebTransfer(H,k,'ring') on the host copy
                for (sp, src, dst) in lev.ops[p]['ring']:
                    lev.QC[p].ravel(order='F')[dst] = H.lev[k - 1].Q[sp - 1].ravel(order='F')[src]
            for p in range(lev.np):
                for cs, vals in _face_corrections(H, k, p):
                    for (dp, src, dst) in cs['ops']:
                        FT = H.lev[k - 1].FTrue[dp - 1].ravel(order='F').copy()
                        FT[dst] = FT[dst] + vals[src]
                        H.lev[k - 1].FTrue[dp - 1] = FT.reshape(H.lev[k - 1].FTrue[dp - 1].shape, order='F')
        H.mark_dirty('QC')
    H.mark_dirty('FTrue')
    return H


def ebpSetTime(H, pprob, t, aDt, force=False):
    """``ebpSetTime.m:11-55``: coefficients, reaction + alpha/Dt, boundary
    data at time t, then fill-down, parent coefficients and the coarsest
    operator; a no-op while the state key is unchanged."""
    td = pprob.tdD or pprob.tdC or pprob.tdBC
    key = (t * td, aDt)
    if not force and H.par.get('stateKey') == key:
        return H
    dom = pprob.domain
    for k in range(1, H.nlev + 1):
        lev = H.lev[k]
        hx, hy = lev.h
        for p in range(lev.np):
            b = lev.box[p]
            xc = dom[0] + (np.arange(b[0], b[1] + 1) - 0.5) * hx
            yc = dom[2] + (np.arange(b[2], b[3] + 1) - 0.5) * hy
            if pprob.tdD or force:
                xf = dom[0] + np.arange(b[0] - 1, b[1] + 1) * hx
                yf = dom[2] + np.arange(b[2] - 1, b[3] + 1) * hy
                XF, YC = np.meshgrid(xf, yc, indexing='ij')
                lev.DeW[p] = np.asfortranarray(np.broadcast_to(pprob.D(XF, YC, t), XF.shape), dtype=float)
                XC, YF = np.meshgrid(xc, yf, indexing='ij')
                lev.DnS[p] = np.asfortranarray(np.broadcast_to(pprob.D(XC, YF, t), XC.shape), dtype=float)
            X, Y = np.meshgrid(xc, yc, indexing='ij')
            lev.CC[p] = np.asfortranarray(np.broadcast_to(pprob.C(X, Y, t), X.shape), dtype=float) + aDt
            if pprob.tdBC or force:
                fint = lev.faceInternal[p]
                bcd = lev.bc[p]
                if not fint[0]:
                    bcd[0]['g'] = np.asarray(pprob.bc[0]['g'](dom[0] * np.ones(yc.shape), yc, t), float).ravel()
                if not fint[1]:
                    bcd[1]['g'] = np.asarray(pprob.bc[1]['g'](dom[1] * np.ones(yc.shape), yc, t), float).ravel()
                if not fint[2]:
                    bcd[2]['g'] = np.asarray(pprob.bc[2]['g'](xc, dom[2] * np.ones(xc.shape), t), float).ravel()
                if not fint[3]:
                    bcd[3]['g'] = np.asarray(pprob.bc[3]['g'](xc, dom[3] * np.ones(xc.shape), t), float).ravel()
    hier.coeff_filldown(H)
    hier.gather_parent_coeffs(H)
    hier.coarsest_assemble(H)
    H.par['stateKey'] = key
    H.par['aDt'] = aDt
    # same hierarchy, new coefficients: an incremental upload, no new plan
    H.mark_dirty('coef')
    return H


def _conslin(W):
    """Conservative linear prolongation with central slopes (``ebpRegrid.m:99-112``)."""
    C0 = W[1:-1, 1:-1]
    sx = (W[2:, 1:-1] - W[:-2, 1:-1]) / 2
    sy = (W[1:-1, 2:] - W[1:-1, :-2]) / 2
    cm, cn = C0.shape
    F = np.zeros((2 * cm, 2 * cn), order='F')
    F[0::2, 0::2] = (C0 - sx / 4) - sy / 4
    F[1::2, 0::2] = (C0 + sx / 4) - sy / 4
    F[0::2, 1::2] = (C0 - sx / 4) + sy / 4
    F[1::2, 1::2] = (C0 + sx / 4) + sy / 4
    return F


def _conslin_interior(P):
    """One-sided slopes at the footprint edges (``ebpRegrid.m:115-137``)."""
    cm, cn = P.shape
    sx = np.zeros((cm, cn))
    sy = np.zeros((cm, cn))
    if cm > 1:
        sx[1:-1, :] = (P[2:, :] - P[:-2, :]) / 2
        sx[0, :] = P[1, :] - P[0, :]
        sx[-1, :] = P[-1, :] - P[-2, :]
    if cn > 1:
        sy[:, 1:-1] = (P[:, 2:] - P[:, :-2]) / 2
        sy[:, 0] = P[:, 1] - P[:, 0]
        sy[:, -1] = P[:, -1] - P[:, -2]
    F = np.zeros((2 * cm, 2 * cn), order='F')
    F[0::2, 0::2] = (P - sx / 4) - sy / 4
    F[1::2, 0::2] = (P + sx / 4) - sy / 4
    F[0::2, 1::2] = (P - sx / 4) + sy / 4
    F[1::2, 1::2] = (P + sx / 4) + sy / 4
    return F


def _gather_window(H, k, p):
    """``ebGatherWindow.m:7-18``: the parent window (ring + interior)."""
    lev = H.lev[k]
    b = lev.box[p]
    cm, cn = (b[1] - b[0] + 1) // 2, (b[3] - b[2] + 1) // 2
    W = np.zeros((cm + 2, cn + 2), order='F')
    ops = lev.ops[p]
    Wf = W.ravel(order='F')
    for (sp, src, dst) in ops['ring']:
        Wf[dst] = H.lev[k - 1].Q[sp - 1].ravel(order='F')[src]
    W = Wf.reshape(W.shape, order='F')
    for (sp, sr, dr) in ops['winrect']:
        W[dr[0] - 1:dr[1], dr[2] - 1:dr[3]] = H.lev[k - 1].Q[sp - 1][sr[0] - 1:sr[1], sr[2] - 1:sr[3]]
    return W


def regrid_keeps(H, pprob, aDtNext, backend):
    """True when ``ebpRegrid`` would rebuild H itself, so the rebuild can be
    skipped with every bit of the state unchanged: H is its root level alone,
    the problem's D, C and boundary data do not depend on time, alpha/Dt is
    the one H's coefficients carry, and tagging H's root marks nothing.  The
    rebuild would then copy H's root solution, restrict it below the root as
    the last fill-down did, sample the same coefficients with the same alpha/Dt
    and add no level (``ebpRegrid.m:16-59``)."""
    if pprob.tdD or pprob.tdC or pprob.tdBC:
        return False
    if H.nlev != H.rootIdx or H.par.get('aDt') != aDtNext:
        return False
    return tag_cluster(H, backend).shape[0] == 0


def history_sources(Hn, fln, Hold, flo):
    """For every cell of the new hierarchy's flat tables at or above its
    root: the old hierarchy's flat cell that holds the same cell of the same
    level (the overwrite of ebpRegrid.m:73-90; the root copies itself,
    :22-26), or -1 where no old patch covers it."""
    from .flat import PD_COFF, PD_MX
    src = np.full(fln.F.size, -1, dtype=np.int32)
    for k in range(Hn.rootIdx, Hn.nlev + 1):
        if k > Hold.nlev:
            break
        for p in range(Hn.lev[k].np):
            b = [int(v) for v in Hn.lev[k].box[p]]
            rn = fln.patches[fln.pglob[(k, p)]]
            con, mxn = int(rn[PD_COFF]), int(rn[PD_MX])
            for q in range(Hold.lev[k].np):
                qb = [int(v) for v in Hold.lev[k].box[q]]
                r = [max(b[0], qb[0]), min(b[1], qb[1]), max(b[2], qb[2]), min(b[3], qb[3])]
                if r[0] > r[1] or r[2] > r[3]:
                    continue
                ro = flo.patches[flo.pglob[(k, q)]]
                coo, mxo = int(ro[PD_COFF]), int(ro[PD_MX])
                i, j = np.meshgrid(np.arange(r[0], r[1] + 1), np.arange(r[2], r[3] + 1), indexing='ij')
                src[con + (i - b[0]) + (j - b[2]) * mxn] = coo + (i - qb[0]) + (j - qb[2]) * mxo
    return src


def ebpRegrid(Hold, pprob, t, aDtNext, opts, backend, history='host'):
    """``ebpRegrid.m:16-59``: new hierarchy on the current solution, with a
    conservative transfer of u and the BDF2 history.  history='device': the
    history stays where it is (resident on the device); the caller moves it
    with the backend's history_transfer once the new hierarchy is built, and
    the returned hierarchy carries no host copy of it."""
    Hn = hier.setup(ebpEprob(pprob, t, aDtNext), opts.eb, backend)
    have_uoo = Hold.par['Uoo'] is not None and history == 'host'
    r = Hn.rootIdx
    Hn.lev[r].Q[0][1:-1, 1:-1] = Hold.lev[r].Q[0][1:-1, 1:-1]
    uoo_n = {}
    if have_uoo:
        uoo_n[(r, 0)] = Hold.par['Uoo'][(r, 0)]
    for k in range(r - 1, 0, -1):
        Hn.lev[k].Q[0][1:-1, 1:-1] = hier.restrict2(Hn.lev[k + 1].Q[0][1:-1, 1:-1])
    Hn.mark_dirty('Q')
    backend.run(Hn, [('fill', k) for k in range(1, r + 1)])
    while (Hn.nlev - Hn.rootIdx + 1) < opts.eb.MaxLevels:
        boxes = tag_cluster(Hn, backend)
        if boxes.shape[0] == 0:
            break
        Hn = hier.add_level(Hn, boxes, backend)
        kN = Hn.nlev
        lev = Hn.lev[kN]
        for p in range(lev.np):
            W = _gather_window(Hn, kN, p)
            Qf = _conslin(W)
            b = [int(v) for v in lev.box[p]]
            cmx, cmy = (b[1] - b[0] + 1) // 2, (b[3] - b[2] + 1) // 2
            if have_uoo:
                Pf = np.zeros((cmx, cmy), order='F')
                for (dp, sr, dr) in lev.ops[p]['fsc']:
                    Pf[sr[0] - 1:sr[1], sr[2] - 1:sr[3]] = uoo_n[(kN - 1, dp - 1)][dr[0] - 1:dr[1], dr[2] - 1:dr[3]]
                Uf = _conslin_interior(Pf)
            if kN <= Hold.nlev:
                for q in range(Hold.lev[kN].np):
                    qb = [int(v) for v in Hold.lev[kN].box[q]]
                    rr = [max(b[0], qb[0]), min(b[1], qb[1]), max(b[2], qb[2]), min(b[3], qb[3])]
                    if rr[0] > rr[1] or rr[2] > rr[3]:
                        continue
                    di = slice(rr[0] - b[0], rr[1] - b[0] + 1)
                    dj = slice(rr[2] - b[2], rr[3] - b[2] + 1)
                    si = slice(rr[0] - qb[0], rr[1] - qb[0] + 1)
                    sj = slice(rr[2] - qb[2], rr[3] - qb[2] + 1)
                    Qf[di, dj] = Hold.lev[kN].Q[q][1:-1, 1:-1][si, sj]
                    if have_uoo:
                        Uf[di, dj] = Hold.par['Uoo'][(kN, q)][si, sj]
            lev.Q[p][1:-1, 1:-1] = Qf
            if have_uoo:
                uoo_n[(kN, p)] = Uf
        Hn.mark_dirty('Q')
        backend.run(Hn, [('fill', kN)])
    backend.run(Hn, [('filldown',)])
    td = pprob.tdD or pprob.tdC or pprob.tdBC
    Hn.par = {'Uo': _interiors(Hn) if history == 'host' else None, 'Uoo': uoo_n if have_uoo else None,
              'stateKey': (t * td, aDtNext), 'aDt': aDtNext}
    Hn.stats = Hold.stats
    return Hn


def _alpha(s):
    return {'be': 1.0, 'bdf2': 1.5, 'cn': 2.0}[s]


def ebpSolve(pprob, *args, backend=None, **kwargs):
    """``ebpSolve.m:17-100``: implicit time stepping with periodic regrids."""
    if len(args) == 1 and isinstance(args[0], dict) and not kwargs:
        opts = args[0]
    else:
        opts = ebpOptions(*args, **kwargs)
    backend = backend or default_backend(opts.eb)
    nsteps = max(1, int(round(opts.TFinal / opts.Dt)))
    Dt = opts.TFinal / nsteps
    scheme1 = 'be' if opts.Scheme == 'bdf2' else opts.Scheme
    H = ebpInit(pprob, opts, _alpha(scheme1) / Dt, backend)
    # a device backend keeps the solution, the source and the BDF2 history
    # resident between steps; they come to the host only for a regrid, a
    # callback, a Crank-Nicolson right-hand side and the result
    dev = getattr(backend, 'resident', False)

    def to_device(H):
        H.par['resident'] = True
        backend.history_set(H, H.par['Uo'], H.par['Uoo'])

    def to_host(H):
        backend.sync_host(H)
        H.par['Uo'], uoo = backend.history_get(H)
        H.par['Uoo'] = uoo if H.par.get('hasUoo') else None
        H.par['resident'] = False

    if dev:
        to_device(H)

    def comp_mass(H):
        m, vol = backend.composite_mean(H)
        return m * vol

    mass = np.zeros(nsteps + 1)
    mass[0] = comp_mass(H)
    cycles = np.zeros(nsteps, dtype=np.int64)
    relres = np.zeros(nsteps)
    nregrids = 0
    for n in range(1, nsteps + 1):
        t1 = n * Dt
        scheme = scheme1 if n == 1 else opts.Scheme
        if dev and scheme in ('be', 'bdf2'):
            fp = None
            if not pprob.get('fzero'):
                fp = {(k, p): pprob.f(*_centres(H, k, p), t1) for k in range(H.rootIdx, H.nlev + 1)
                      for p in range(H.lev[k].np)}
                fp = {kp: np.broadcast_to(v, _centres(H, *kp)[0].shape) for kp, v in fp.items()}
            backend.parabolic_rhs(H, scheme, Dt, fp)
        elif dev:
            to_host(H)
            H = ebpRhs(H, pprob, t1, Dt, scheme, backend)
            to_device(H)
        else:
            H = ebpRhs(H, pprob, t1, Dt, scheme, backend)
        H = ebpSetTime(H, pprob, t1, _alpha(scheme) / Dt)
        H = ebSolveCycles(H, backend)
        st = H.stats['stages'][-1]
        cycles[n - 1] = st['vcycles']
        relres[n - 1] = st['finalRel']
        if dev:
            backend.history_push(H)
            H.par['hasUoo'] = True
        else:
            H.par['Uoo'] = H.par['Uo']
            H.par['Uo'] = _interiors(H)
        mass[n] = comp_mass(H)
        if opts.Callback is not None:
            if dev:
                to_host(H)
                opts.Callback(H, t1, n)
                to_device(H)
            else:
                opts.Callback(H, t1, n)
        sv = int(opts.StepVerbose)
        if sv > 0 and (n % sv == 0 or n == nsteps):
            nc = sum(f.size for k in range(H.rootIdx, H.nlev + 1) for f in H.lev[k].FTrue)
            print(f'[ebsam-p] step {n:4d}/{nsteps}  t={t1:.4f}  V={cycles[n - 1]}  rel={relres[n - 1]:.1e}  '
                  f'levels={H.nlev - H.rootIdx + 1}  cells={nc}  mass={mass[n]:.6e}')
        if opts.RegridEvery > 0 and n % int(opts.RegridEvery) == 0 and n < nsteps and opts.eb.MaxLevels > 1:
            aNext = _alpha(opts.Scheme) / Dt
            if dev:
                # the solution comes to the host for the new hierarchy's
                # build (tagging, conservative transfer of u); the BDF2
                # history moves device to device
                backend.sync_host(H)
                if not regrid_keeps(H, pprob, aNext, backend):
                    Hold = H
                    H = ebpRegrid(Hold, pprob, t1, aNext, opts, backend, history='device')
                    H.par['resident'] = True
                    H.par['hasUoo'] = bool(Hold.par.get('hasUoo'))
                    backend.history_transfer(H, Hold, H.par['hasUoo'])
                    del Hold
            elif not regrid_keeps(H, pprob, aNext, backend):
                H = ebpRegrid(H, pprob, t1, aNext, opts, backend)
            nregrids += 1
    if dev:
        to_host(H)
    sol = {'H': H, 't': np.arange(nsteps + 1) * Dt, 'mass': mass, 'cycles': cycles, 'relres': relres,
           'nregrids': nregrids, 'stats': H.stats}
    if pprob.exact is not None:
        T = opts.TFinal
        sol['err'] = error_norms(H, lambda x, y: pprob.exact(x, y, T))
    else:
        sol['err'] = None
    sol['levels'] = [{'n': H.lev[k].n, 'np': H.lev[k].np, 'cells': sum(f.size for f in H.lev[k].FTrue)}
                     for k in range(H.rootIdx, H.nlev + 1)]
    return sol
