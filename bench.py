"""Benchmark: the diffuse-domain starfish solve (BSAM-in-MATLAB examples/
demoStarfish.m 'full': 64^2 base refined through 5 AMR levels to 1024^2-
equivalent spacing, 543,384 stored cells, RelTol 1e-10) on one GB300.

One step = one ebSolveCycles of that hierarchy from its initial state (zero
initial guess): ghost fill, initial residual, V(3,3)-cycles to relative
composite residual 1e-10 (10 cycles).

  value   solves/s with the hierarchy resident in HBM (device-side state
          restore before each solve; L2 flushed between solves by writing a
          256 MiB buffer, the hierarchy being ~40 MB).
  e2e     the same solves through the C-ABI with host buffers: per solve the
          initial guess and source go host->device, the solution and the
          residual history come back (pinned host memory).
  roofline  the red-black smoother on the finest level (the dominant kernel),
          algorithmic bytes 48 B per cell per red+black sweep (24 B per colour
          pass), per-launch CUDA-event times of eagerly launched V-cycles, on
          the library's stream, against the measured HBM copy peak; `traffic`
          is the DRAM bytes per launch of the same launch from the committed
          ncu summary (profiles/k_relax_starfish_finest.md).
  cpu_baseline  the C oracle (a restatement of the reference's MATLAB path)
          on the host cores, a bounded sample of whole solves.

  forms   beside the plain FP64 path (same JSON line, key "forms"):
          mixed   the starfish solve in the mixed-precision form (FP32
                  correction V-cycles inside FP64 defect correction, same FP64
                  stop test), with its relative L2 / max difference from the
                  FP64 solution;
          batched 256 seeded random elliptic instances (BaseCells {32,64,128},
                  MaxLevels {2,3,4}, TagThreshold 1e-2), the last ebSolve stage
                  of each: solved one after another on the plain path, then as
                  one batch in FP64 (checked bit for bit against the solo
                  solves) and in the mixed form;
          serving Poisson streams of diffuse-domain star requests at a few
                  offered rates through the continuous-batching server
                  (bsam.serve): solves/s and p50/p99 latency.

`--impl reference` times the reference's CPU path instead: MATLAB is not
available, so the C oracle restatement runs on all host cores.
With several GPUs (`--gpus N`: the script starts N ranks under
torch.distributed.run unless it already runs under it) every rank solves its
own replica of the starfish -- the hierarchy does not shard -- and the
batching form's instances shard by instance across the ranks; neither has a
data-path collective, and every rate is the units of all ranks over the
slowest rank's time.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, 'bsam-in-matlab_gb300'), os.path.join(ROOT, 'oracle')):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = 'solves/s & p50/p99 ms at rel resid 1e-10, mixed vs FP64 GPU; smoother HBM GB/s'
WORKLOAD = ('starfish diffuse-domain transmission, 64^2 base + 5 AMR levels (1024^2-equivalent), '
            '543384 stored cells, QC-ring hierarchy, V(3,3), RelTol 1e-10, FP64')


def starfish_hierarchy(backend):
    from bsam import ebOptions
    from bsam.ddm import starfish_problem, starfish_tag
    from bsam.solve import build_hierarchy
    prob, aux, g = starfish_problem()
    opts = ebOptions('BaseCells', 64, 'MaxLevels', 5, 'Indicator', 'fun', 'TagFunction', starfish_tag(g),
                     'TagBuffer', 2, 'RelTol', 1e-10, 'MaxVCycles', 100, 'Verbose', 0)
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        H = build_hierarchy(prob, opts, backend)
    return H, opts


def load_traffic():
    """DRAM bytes per finest-level smoother launch from the committed ncu summary."""
    import re
    p = os.path.join(ROOT, 'profiles', 'k_relax_starfish_finest.md')
    if not os.path.exists(p):
        return None
    m = re.search(r'dram_bytes_per_launch:\s*([0-9.eE+]+)', open(p).read())
    return float(m.group(1)) if m else None


def load_peaks():
    p = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d['hbm_gbs']), 'measured'
    return 6800.0, 'fallback'


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs: the
    sampler starts before the region (it waits for its first sample, so the
    tool's start-up falls outside), samples every 20 ms, and keeps the
    samples that arrive between mark_start() and mark_end()."""

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None
        self.t0 = self.t1 = None

    def __enter__(self):
        q = ('clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,'
             'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,'
             'clocks_event_reasons.sw_power_cap')
        try:
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.index), f'--query-gpu={q}',
                                          '--format=csv,noheader,nounits', '-lms', '20'],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            deadline = time.perf_counter() + 5.0
            while not self.rows and time.perf_counter() < deadline and self.proc.poll() is None:
                time.sleep(0.01)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [s.strip() for s in line.split(',')]
            if len(parts) == 7:
                self.rows.append((time.perf_counter(), parts))

    def mark_start(self):
        self.t0 = time.perf_counter()

    def mark_end(self):
        self.t1 = time.perf_counter()
        time.sleep(0.05)          # the sample of the region's last moments

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['unsampled']}
        t0 = self.t0 if self.t0 is not None else -1e30
        t1 = (self.t1 + 0.04) if self.t1 is not None else 1e30
        inside = [r for t, r in self.rows if t0 <= t <= t1]
        rows = inside or [r for _, r in self.rows]
        sm = [float(r[0]) for r in rows if r[0].replace('.', '').isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace('.', '').isdigit()]
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        reasons = sorted({names[i] for r in rows for i in range(4) if r[3 + i].lower() == 'active'})
        return {'sm_mhz': float(np.median(sm)) if sm else None, 'sm_max_mhz': max(mx) if mx else None,
                'reasons': reasons, 'samples': len(rows), 'in_region': bool(inside)}


def cpu_oracle_rate(H, opts, threads, budget_s):
    """Solves/s of the C oracle on `threads` host threads (bounded sample)."""
    os.environ['OMP_NUM_THREADS'] = str(threads)
    from bsam.flat import flatten
    from bsam_oracle import OracleHier
    fl = flatten(H)
    n = 0
    t0 = time.perf_counter()
    while True:
        oh = OracleHier(fl, opts)
        it, hist, rel, vis = oh.solve_cycles(opts.MaxVCycles + 2)
        n += 1
        el = time.perf_counter() - t0
        if el >= budget_s or n >= 50:
            break
    return n / el, n, el, it, rel


def run_reference(args, rank, world):
    """--impl reference: the reference's CPU path (C oracle restatement; MATLAB
    is not installed) on all host threads, same workload and metric."""
    if rank != 0:
        return
    from bsam_oracle import OracleBackend, build as build_oracle
    build_oracle()
    H, opts = starfish_hierarchy(OracleBackend())
    threads = os.cpu_count() or 1
    os.environ['OMP_NUM_THREADS'] = str(threads)
    from bsam.flat import flatten
    from bsam_oracle import OracleHier
    fl = flatten(H)
    times = []
    for s in range(args.warmup + args.steps):
        oh = OracleHier(fl, opts)
        t0 = time.perf_counter()
        it, hist, rel, vis = oh.solve_cycles(opts.MaxVCycles + 2)
        dt = time.perf_counter() - t0
        if s >= args.warmup:
            times.append(dt)
    tot = sum(times)
    value = len(times) / tot
    line = {'metric': METRIC, 'value': value, 'unit': 'solves/s', 'n_gpus': world, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': 1e3 * tot / len(times), 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic',
            'impl': 'reference',
            'config': {'workload': WORKLOAD, 'vcycles': it, 'final_rel': rel},
            'cpu_baseline': {'value': value, 'unit': 'solves/s', 'cores': threads, 'kind': 'port',
                             'sample': f'{len(times)} full starfish solves (MATLAB absent: C oracle restatement)'},
            'e2e': {'value': value, 'unit': 'solves/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line), flush=True)


def time_device_solves(dh, opts, steps, warmup, stream, flush):
    """Per-solve device times (CUDA events on the library stream, L2
    flushed before each solve, state restored on the device)."""
    import torch
    dh.save_state()
    for _ in range(warmup):
        dh.restore_state()
        r = dh.solve_cycles(opts.MaxVCycles + 2)
    ms = []
    for _ in range(steps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            flush.zero_()
            a.record(stream)
        dh.restore_state()
        r = dh.solve_cycles(opts.MaxVCycles + 2)
        b.record(stream)
        torch.cuda.synchronize()
        ms.append(a.elapsed_time(b))
    return np.array(ms), r


def mixed_form(backend, fl, opts, ref_Q, steps, warmup, flush, local):
    """Precision form on the starfish hierarchy: FP32 correction cycles in
    an FP64 defect-correction loop, to the same FP64 stop test."""
    import torch
    from bsam.device import DevHier, BSAM_FIELD_Q
    from bsam.flat import visible_q_index, rel_errors
    om = opts.copy()
    om['Precision'] = 'mixed'
    dh = DevHier(backend.ctx, fl, om)
    stream = torch.cuda.ExternalStream(dh.stream(), device=torch.device('cuda', local))
    ms, r = time_device_solves(dh, om, steps, warmup, stream, flush)
    l2, mx = rel_errors(dh.get(BSAM_FIELD_Q, fl.Q.size), ref_Q, visible_q_index(fl))
    return {'value': steps / (ms.sum() / 1e3), 'unit': 'solves/s', 'ms_per_solve': float(ms.mean()),
            'p50_ms': float(np.percentile(ms, 50)), 'p99_ms': float(np.percentile(ms, 99)),
            'vcycles': r[0], 'final_rel': r[2], 'rel_l2_vs_fp64': l2, 'rel_max_vs_fp64': mx,
            'relax_cells_per_thread': dh.relax_tuning(1).tolist(), 'kernels_per_vcycle': dh.kernels_per_vcycle(),
            'dtype': 'f32 smoothing / f64 defect correction',
            'note': 'error against the FP64 path, which equals the C oracle bit for bit'}


def batched_form(backend, n, steps, warmup, flush, local, dist=None):
    """Batching form: n seeded random elliptic instances (BaseCells
    {32,64,128}, MaxLevels {2,3,4}, TagThreshold 1e-2), each taken through
    ebSolve's solution-driven pipeline to its last stage; that last solve of
    every instance runs (a) alone, one after another (the plain FP64 path),
    (b) as one batch in FP64, (c) as one batch in the mixed form.  With
    several ranks the instances shard by instance (rank r takes instances
    r, r + N, ...), each rank batching its own share with no collective; the
    rates count every rank's instances over the slowest rank's time."""
    import torch
    import warnings
    from bsam.device import DevHier, BSAM_FIELD_Q
    from bsam.instances import random_elliptic, final_stage
    from bsam.batch import merge_flats, split_field
    from bsam.flat import FIELD_Q, visible_q_index, rel_errors
    from bsam.replicas import shard, job_rate_units, gather
    rank = dist.get_rank() if dist else 0
    world = dist.get_world_size() if dist else 1
    ids = shard(n, rank, world)
    dev = torch.device('cuda', local)
    t0 = time.perf_counter()
    parts, opts = [], None
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        for s in ids:
            prob, o = random_elliptic(1000 + s)
            fl, H = final_stage(prob, o, backend)
            parts.append(fl)
            opts = opts or H.opts
    setup_s = time.perf_counter() - t0
    # (a) solo, plain FP64
    solo_ms, solo = [], []
    for p in parts:
        dh = DevHier(backend.ctx, p, opts)
        st = torch.cuda.ExternalStream(dh.stream(), device=dev)
        ms, r = time_device_solves(dh, opts, 1, 1, st, flush)
        solo_ms.append(float(ms[0]))
        solo.append((r, dh.get(BSAM_FIELD_Q, p.Q.size)))
        del dh
    solo_total = sum(solo_ms)
    solo_rate, solo_t = job_rate_units(len(ids), solo_total / 1e3, dist, dev)
    all_solo = [v for r in gather(solo_ms, dist) for v in r]
    out = {'workload': f'{n} seeded random elliptic instances on [0,1]^2 (log D: 16 Fourier modes, C in [0,1], '
                       f'f: 4 Gaussian bumps; BaseCells {{32,64,128}}, MaxLevels {{2,3,4}}, TagThreshold 1e-2), '
                       f'last ebSolve stage of each, RelTol 1e-10',
           'instances': n, 'ranks': world, 'instances_per_rank': [len(shard(n, r, world)) for r in range(world)],
           'stored_cells': int(sum(gather(int(sum(p.F.size for p in parts)), dist))), 'setup_s': setup_s,
           'solo_fp64': {'value': solo_rate, 'unit': 'solves/s', 'ms_total': 1e3 * solo_t,
                         'p50_ms': float(np.percentile(all_solo, 50)), 'p99_ms': float(np.percentile(all_solo, 99))}}
    b = merge_flats(parts)
    for prec in ('fp64', 'mixed'):
        ob = opts.copy()
        ob['Precision'] = prec
        bh = DevHier(backend.ctx, b, ob)
        st = torch.cuda.ExternalStream(bh.stream(), device=dev)
        ms, _ = time_device_solves(bh, ob, steps, warmup, st, flush)
        Q = bh.get(BSAM_FIELD_Q, b.Q.size)
        equal, worst_l2, worst_max, maxit = True, 0.0, 0.0, 0
        for i, (r, q) in enumerate(solo):
            rb = bh.batch_result(i, ob.MaxVCycles + 2)
            maxit = max(maxit, rb[0])
            qi = split_field(b, FIELD_Q, Q, i)
            if prec == 'fp64':
                equal &= rb[0] == r[0] and np.array_equal(rb[1], r[1]) and np.array_equal(qi, q)
            else:
                l2, mx = rel_errors(qi, q, visible_q_index(parts[i]))
                worst_l2, worst_max = max(worst_l2, l2), max(worst_max, mx)
        rate, tmax = job_rate_units(len(ids) * steps, ms.sum() / 1e3, dist, dev)
        equal = all(gather(bool(equal), dist))
        maxit = max(gather(maxit, dist))
        worst_l2, worst_max = max(gather(worst_l2, dist)), max(gather(worst_max, dist))
        d = {'value': rate, 'unit': 'solves/s', 'ms_per_batch': 1e3 * tmax / steps,
             'p50_ms': float(np.percentile(ms, 50)), 'p99_ms': float(np.percentile(ms, 99)),
             'vcycles_slowest': maxit, 'kernels_per_vcycle': bh.kernels_per_vcycle(),
             'relax_cells_per_thread': bh.relax_tuning(1 if prec == 'mixed' else 0).tolist()}
        # smoother roofline per merged level (levels larger than L2 here)
        peak, peak_kind = load_peaks()
        from bsam.device import fp64_rate
        fp64_peak = fp64_rate(backend.ctx)
        cells = [int(b.levels[k - 1, 5] - b.levels[k - 1, 4]) for k in range(1, b.nlev + 1)]
        lv = []
        for k in range(2, b.nlev + 1):
            pr = bh.profile(2, level=k)['relax']
            if pr['launches']:
                ach = pr['bytes'] / (pr['ms'] / 1e3) / 1e9
                us = 1e3 * pr['ms'] / pr['launches']
                lv.append({'level': k, 'cells': cells[k - 1], 'avg_launch_us': us,
                           'achieved_gbs': ach, 'frac': ach / peak})
                if prec == 'fp64':   # 9 FP64 operations per 48 algorithmic bytes
                    lv[-1]['fp64_pipe_frac'] = pr['bytes'] * 9 / 48 / (pr['ms'] / 1e3) / 1e9 / fp64_peak
        d['smoother_levels'] = lv
        d['smoother_peak'] = {'value': peak, 'kind': peak_kind, 'unit': 'GB/s'}
        if prec == 'fp64':
            d['equal_to_solo_bitwise'] = bool(equal)
        else:
            d['worst_rel_l2_vs_fp64'] = worst_l2
            d['worst_rel_max_vs_fp64'] = worst_max
        out['batch_' + prec] = d
        del bh
    out['speedup_batch_mixed_vs_solo_fp64'] = out['batch_mixed']['value'] / out['solo_fp64']['value']
    return out


def serving_form(rates, per_rate):
    """Serving form: Poisson streams of diffuse-domain star requests (k in
    {3..7}, b, a0, theta0, eps drawn per request, base 64^2, MaxLevels
    {3,4,5}, mixed precision, RelTol 1e-10) through the continuous-batching
    server; p50/p99 latency from submission to the solution on the host."""
    from bsam.serve import Server, star_request, run_stream, summarize
    t0 = time.perf_counter()
    srv = Server(waves=3, wave_size=64)
    start_s = time.perf_counter() - t0
    warm, _ = run_stream(srv, [star_request(90000 + i) for i in range(srv.nbuild)], rate=100.0, seed=9)
    out = {'workload': 'served diffuse-domain star requests (Poisson arrivals), base 64^2, MaxLevels U{3,4,5}, '
                       'mixed precision, RelTol 1e-10',
           'builders': srv.nbuild, 'wave_slots': len(srv.ctxs), 'server_start_s': start_s, 'rates': [],
           'gpu_distance': srv.distance is not None}
    for rate in rates:
        # about four seconds of arrivals, 30 to 120 requests: enough to see
        # where the delivered rate stops following the offered one
        n = int(min(max(per_rate, round(rate * 4)), 120))
        specs = [star_request(int(rate * 1000) + i) for i in range(n)]
        w0 = len(srv.waves_run)
        res, wall = run_stream(srv, specs, rate=rate, seed=int(rate))
        d = summarize(res, wall)
        d['offered_rate'] = rate
        sizes = [w['size'] for w in srv.waves_run[w0:]]
        d['waves'] = len(sizes)
        d['mean_wave_size'] = float(np.mean(sizes)) if sizes else 0.0
        out['rates'].append(d)
    # a mixed stream: one request in four is a parabolic run (BDF2 heat,
    # 10 steps with regrids) holding a wave slot for its whole run
    from bsam.serve import heat_request
    rate = 10.0
    specs = [heat_request(50000 + i) if i % 4 == 3 else star_request(60000 + i) for i in range(40)]
    res, wall = run_stream(srv, specs, rate=rate, seed=77)
    d = summarize(res, wall)
    d['offered_rate'] = rate
    d['parabolic_share'] = 0.25
    par = [r for r in res if r.spec.get('kind') == 'parabolic']
    d['parabolic_p50_ms'] = float(np.percentile([r.latency_s * 1e3 for r in par], 50))
    out['mixed_stream'] = d
    srv.close()
    if srv.distance is not None:
        out['distance_service'] = {'calls': srv.distance.calls, 'points': srv.distance.points,
                                   'busy_s': srv.distance.busy_s}
    ok = [r for r in out['rates']]
    if ok:
        best = max(ok, key=lambda r: r['solves_per_s'])
        out['saturation'] = {'offered_rate': best['offered_rate'], 'solves_per_s': best['solves_per_s'],
                             'mean_wave_size': best['mean_wave_size']}
    return out


def parabolic_form(backend):
    """Config 3: the README heat example (BDF2, Dt 0.002, TFinal 0.1,
    RegridEvery 5) at BaseCells 32 / MaxLevels 3 and 128 / MaxLevels 4, with
    the solution, source and BDF2 history resident on the device between
    steps; composite mass drift per step."""
    from bsam.parabolic import ebpProblem, ebpSolve
    u0 = lambda x, y: 1 + 0.2 * np.cos(2 * np.pi * x) * np.cos(2 * np.pi * y)
    prob = ebpProblem([0, 1, 0, 1], 1, 0, 0, ('neumann', 0), u0)
    out = []
    for base, ml in ((32, 3), (128, 4)):
        t0 = time.perf_counter()
        sol = ebpSolve(prob, 'Scheme', 'bdf2', 'Dt', 0.002, 'TFinal', 0.1, 'BaseCells', base, 'MaxLevels', ml,
                       'RegridEvery', 5, 'StepVerbose', 0, backend=backend)
        wall = time.perf_counter() - t0
        m = sol['mass']
        out.append({'BaseCells': base, 'MaxLevels': ml, 'steps': len(sol['cycles']), 'wall_s': wall,
                    'steps_per_s': len(sol['cycles']) / wall, 'vcycles_total': int(np.sum(sol['cycles'])),
                    'max_step_rel': float(np.max(sol['relres'])), 'regrids': sol['nregrids'],
                    'mass_drift_per_step_max': float(np.max(np.abs(np.diff(m)))),
                    'mass_drift_total': float(abs(m[-1] - m[0])),
                    'final_levels': [lv['np'] for lv in sol['levels']]})
    # a run whose hierarchy keeps three levels through every regrid: the
    # reference's rotating-source case (ParabolicBSAM/tests/runParabolicTests.m
    # P3: BDF2, Dt 5e-3, TFinal 1, RegridEvery 4, BaseCells 64, MaxLevels 3,
    # 'ulap' tagging), history moved device to device at each regrid
    import warnings
    from bsam.device import DeviceBackend
    om, Rc, ss = 2 * np.pi, 0.22, 0.03
    src = lambda x, y, t: 25 * np.exp(-((x - (0.5 + Rc * np.cos(om * t))) ** 2 +
                                        (y - (0.5 + Rc * np.sin(om * t))) ** 2) / (2 * ss ** 2))
    p3 = ebpProblem([0, 1, 0, 1], 1, 0, src, ('dirichlet', 0), lambda x, y: 0 * x)
    h0 = DeviceBackend.history_downloads
    t0 = time.perf_counter()
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        sol = ebpSolve(p3, 'Scheme', 'bdf2', 'Dt', 5e-3, 'TFinal', 1.0, 'RegridEvery', 4, 'StepVerbose', 0,
                       'BaseCells', [64, 64], 'MaxLevels', 3, 'Indicator', 'ulap',
                       'TagThreshold', lambda L: 2e-3 / 4 ** (L - 1), 'TagBuffer', 3, 'RelTol', 1e-8,
                       backend=backend)
    wall = time.perf_counter() - t0
    rot = {'workload': 'rotating Gaussian source (P3), BDF2, Dt 5e-3, TFinal 1, RegridEvery 4, BaseCells 64, '
                       'MaxLevels 3, ulap tagging', 'steps': len(sol['cycles']), 'wall_s': wall,
           'steps_per_s': len(sol['cycles']) / wall, 'vcycles_total': int(np.sum(sol['cycles'])),
           'max_step_rel': float(np.max(sol['relres'])), 'regrids': sol['nregrids'],
           'final_levels': [lv['np'] for lv in sol['levels']], 'final_cells': [lv['cells'] for lv in sol['levels']],
           'history_downloads': DeviceBackend.history_downloads - h0}
    return {'workload': 'README heat example, BDF2, Dt 0.002, TFinal 0.1, RegridEvery 5 (wall time includes the '
                        'host regrids)', 'runs': out, 'rotating_source': rot}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=20)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='native', choices=['native', 'reference'])
    ap.add_argument('--cpu-budget', type=float, default=15.0)
    ap.add_argument('--batch', type=int, default=256, help='instances of the batching form (0: skip)')
    ap.add_argument('--no-forms', action='store_true', help='skip the mixed, batching and serving forms')
    ap.add_argument('--serve-rates', default='5,10,20,50,100,200', help='offered request rates of the serving form')
    ap.add_argument('--eager-vcycle', nargs='?', const='fp64', choices=['fp64', 'mixed'],
                    help='profiling aid: upload the starfish hierarchy, solve it once (which tunes the smoother), '
                         'put the initial state back and run one eager V-cycle in that precision (every kernel of '
                         'the V-cycle, fill-down and residual launched once, in order, between cudaProfilerStart and '
                         'cudaProfilerStop) and exit; for ncu --profile-from-start off')
    args = ap.parse_args()
    if 'WORLD_SIZE' not in os.environ and args.gpus > 1 and args.impl == 'native':
        # one process per GPU: start the ranks under torch.distributed.run
        import socket
        sk = socket.socket()
        sk.bind(('127.0.0.1', 0))
        port = sk.getsockname()[1]
        sk.close()
        os.execv(sys.executable, [sys.executable, '-m', 'torch.distributed.run', '--nnodes=1',
                                  f'--nproc-per-node={args.gpus}', '--master-addr', '127.0.0.1',
                                  '--master-port', str(port), os.path.abspath(__file__)] + sys.argv[1:])
    rank = int(os.environ.get('RANK', 0))
    world = int(os.environ.get('WORLD_SIZE', 1))
    local = int(os.environ.get('LOCAL_RANK', 0))
    if args.impl == 'native' and world != args.gpus:
        sys.exit(f'bench.py: --gpus {args.gpus} but WORLD_SIZE is {world}: one rank per GPU is required')
    if args.impl == 'reference':
        return run_reference(args, rank, world)

    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group('nccl')
    from bsam.build import build_all
    build_all()
    from bsam.device import DeviceBackend, DevHier, BSAM_FIELD_Q, BSAM_FIELD_FTRUE, lib, check
    from bsam.flat import flatten
    backend = DeviceBackend.get(local)
    t_setup0 = time.perf_counter()
    H, opts = starfish_hierarchy(backend)
    t_build = time.perf_counter()
    fl = flatten(H)
    if args.eager_vcycle == 'mixed':
        opts['Precision'] = 'mixed'
    dh = DevHier(backend.ctx, fl, opts)
    if args.eager_vcycle:
        dh.save_state()
        dh.solve_cycles(opts.MaxVCycles + 2)
        dh.restore_state()
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        dh.vcycle()
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
        print(json.dumps({'eager_vcycle': 'done', 'precision': args.eager_vcycle, 'levels': H.nlev,
                          'kernels': dh.kernels_per_vcycle(), 'relax_forms': dh.relax_tuning(
                              1 if args.eager_vcycle == 'mixed' else 0).tolist()}), flush=True)
        return
    dh.save_state()
    t_upload = time.perf_counter()
    stream = torch.cuda.ExternalStream(dh.stream(), device=torch.device('cuda', local))
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f'cuda:{local}')

    def one_solve():
        dh.restore_state()
        return dh.solve_cycles(opts.MaxVCycles + 2)

    # warm-up; the first solve also tunes the smoother and captures the
    # V-cycle graph, and ends the set-up-and-solve time of a fresh hierarchy
    it, hist, rel, vis = one_solve()
    t_first = time.perf_counter()
    for _ in range(max(args.warmup - 1, 0)):
        it, hist, rel, vis = one_solve()
    assert rel <= 1e-10, rel

    # ---- device-resident timing ------------------------------------------
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    n0 = dh.launch_count()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        clk.mark_start()
        for s in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
                starts[s].record(stream)
            it, hist, rel, vis = one_solve()
            ends[s].record(stream)
        torch.cuda.synchronize()
        clk.mark_end()
    launches = dh.launch_count() - n0
    per = np.array([a.elapsed_time(b) for a, b in zip(starts, ends)])
    from bsam.replicas import job_rate
    # replicas: the job time is the slowest rank's (no data-path collective)
    value, total_s = job_rate(args.steps, float(per.sum()) / 1e3, dist, torch.device('cuda', local))
    total_ms = 1e3 * total_s

    # ---- end to end through the C-ABI with host buffers ---------------------
    Q0 = torch.from_numpy(fl.Q.copy()).pin_memory().numpy()
    F0 = torch.from_numpy(fl.FTrue.copy()).pin_memory().numpy()
    Qout = torch.empty(fl.Q.size, dtype=torch.float64).pin_memory().numpy()
    hist_bytes = 8 * (opts.MaxVCycles + 2)
    import ctypes as C
    L = lib()
    e2e_ms = []
    torch.cuda.synchronize()
    for s in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dh.restore_state()
        check(L.bsam_set_field(dh.h, BSAM_FIELD_Q, Q0.ctypes.data, Q0.size))
        check(L.bsam_set_field(dh.h, BSAM_FIELD_FTRUE, F0.ctypes.data, F0.size))
        it2, hist2, rel2, _ = dh.solve_cycles(opts.MaxVCycles + 2)
        check(L.bsam_get_field(dh.h, BSAM_FIELD_Q, Qout.ctypes.data, Qout.size))
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    assert rel2 <= 1e-10
    e2e_value, _ = job_rate(args.steps, sum(e2e_ms) / 1e3, dist, torch.device('cuda', local))

    # ---- roofline of the smoother -------------------------------------------
    prof = dh.profile(3)
    fine = dh.profile(3, level=H.nlev)
    peak, peak_kind = load_peaks()
    rl = fine['relax']
    bytes_per_pass = rl['bytes'] / max(rl['launches'], 1)
    eager_us = 1e3 * rl['ms'] / max(rl['launches'], 1)
    # the finest level's colour pass as the solve runs it: the relaxation's
    # passes as one graph of programmatic-launch-chained kernels, replayed
    # with CUDA events on the library's stream (the per-launch event pairs of
    # the eager profile above also time each launch's own overhead)
    pass_us = dh.time_relax(H.nlev, 20)
    dh.restore_state()
    achieved = bytes_per_pass / (pass_us / 1e6) / 1e9
    ra = prof['relax']
    achieved_all = ra['bytes'] / (ra['ms'] / 1e3) / 1e9
    # the FP64 smoother's other bound: 9 separate FP64 operations per colour
    # update (4 products, 4 sums, the diagonal product; no contraction), i.e.
    # 9 per 48 algorithmic bytes (a pass moves 24 B per cell, updates half)
    from bsam.device import fp64_rate
    fp64_peak = fp64_rate(backend.ctx)
    fp64_ach = bytes_per_pass * 9 / 48 / (pass_us / 1e6) / 1e9
    # per kernel kind over all levels: time, launches and the algorithmic
    # bytes of each kind (smoother 24 B per cell and colour pass, coarse load
    # 50, prolongation 20, restriction 12, residual 41; ghost fills and the
    # coarsest solve have none) against the copy peak
    per_kind = {k: {'ms_per_cycle': v['ms'] / 3, 'launches_per_cycle': v['launches'] / 3,
                    'bytes_per_cycle': v['bytes'] / 3,
                    'achieved_gbs': (v['bytes'] / (v['ms'] / 1e3) / 1e9) if v['ms'] > 0 and v['bytes'] > 0 else None,
                    'frac': (v['bytes'] / (v['ms'] / 1e3) / 1e9 / peak) if v['ms'] > 0 and v['bytes'] > 0 else None}
                for k, v in prof.items() if v['launches']}

    # ---- forms beside the plain FP64 path -----------------------------------
    forms = None
    if not args.no_forms:
        dh.restore_state()
        dh.solve_cycles(opts.MaxVCycles + 2)
        ref_Q = dh.get(BSAM_FIELD_Q, fl.Q.size)
        forms = {'mixed': mixed_form(backend, fl, opts, ref_Q, args.steps, args.warmup, flush, local)}
        forms['mixed']['speedup_vs_fp64'] = forms['mixed']['value'] / value
        if args.batch > 0:
            forms['batched'] = batched_form(backend, args.batch, max(3, args.steps // 4), args.warmup, flush, local,
                                            dist)
        forms['parabolic'] = parabolic_form(backend)
        rates = [float(r) for r in args.serve_rates.split(',') if r.strip()]
        if rates and rank == 0:
            forms['serving'] = serving_form(rates, 30)

    if rank == 0:
        cpu = None
        try:
            from bsam_oracle import build as build_oracle
            build_oracle()
            rate, n, el, itc, relc = cpu_oracle_rate(H, opts, 1, args.cpu_budget)
            cpu = {'value': rate, 'unit': 'solves/s', 'cores': 1, 'kind': 'port',
                   'sample': f'{n} full starfish solves on 1 host thread in {el:.1f} s (C oracle restatement; '
                             f'MATLAB not installed)'}
        except Exception as e:  # report, do not hide
            cpu = {'value': None, 'unit': 'solves/s', 'cores': 0, 'kind': 'port', 'sample': f'failed: {e}'}
        line = {
            'metric': METRIC, 'value': value, 'unit': 'solves/s', 'n_gpus': world, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': total_ms / args.steps, 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic',
            'config': {'workload': WORKLOAD, 'parallelism': 'replicas' if world > 1 else 'single',
                       'l2': 'flushed between solves (256 MiB write)', 'vcycles_per_solve': it,
                       'final_rel': rel, 'visible_cells': vis, 'stored_cells': int(fl.F.size - 0),
                       'p50_ms': float(np.percentile(per, 50)), 'p99_ms': float(np.percentile(per, 99)),
                       'kernels_per_vcycle': dh.kernels_per_vcycle(), 'per_kernel': per_kind,
                       'relax_cells_per_thread': dh.relax_tuning(0).tolist()},
            'e2e': {'value': e2e_value, 'unit': 'solves/s',
                    'h2d_bytes_per_step': int(8 * (Q0.size + F0.size)),
                    'd2h_bytes_per_step': int(8 * Qout.size + hist_bytes),
                    'p50_ms': float(np.percentile(e2e_ms, 50)), 'p99_ms': float(np.percentile(e2e_ms, 99))},
            'roofline': {'bound': 'hbm', 'achieved': achieved, 'peak': peak, 'unit': 'GB/s',
                         'frac': achieved / peak, 'traffic': load_traffic(), 'peak_kind': peak_kind,
                         'kernel': f'k_relax, finest level ({fl.levels[H.nlev - 1, 5] - fl.levels[H.nlev - 1, 4]} '
                                   f'cells, one colour pass)',
                         'bytes_per_launch': bytes_per_pass,
                         'avg_launch_us': pass_us,
                         'timing': 'graph replay of the level\'s chained colour passes, CUDA events, per pass',
                         'eager_avg_launch_us': eager_us,
                         'all_levels': {'achieved': achieved_all, 'frac': achieved_all / peak,
                                        'avg_launch_us': 1e3 * ra['ms'] / max(ra['launches'], 1)},
                         'fp64_pipe': {'ops_per_update': 9, 'achieved_gops': fp64_ach, 'peak_gops': fp64_peak,
                                       'peak_kind': 'measured (bsam_fp64_rate)', 'frac': fp64_ach / fp64_peak}},
            'cpu_baseline': cpu,
            # a fresh starfish from problem to converged solution: host build
            # (geometry, coefficients, tagging, clustering, the set-up's device
            # fills), flatten + upload, first solve (tuning and graph capture
            # included); the reference records 11.07 s for its set-up and solve
            # of the same hierarchy (verification/starfish-full.json,
            # setupAndSolveSeconds, MATLAB R2026a on its own machine)
            'setup': {'host_build_s': t_build - t_setup0, 'flatten_upload_s': t_upload - t_build,
                      'first_solve_s': t_first - t_upload, 'setup_and_solve_s': t_first - t_setup0,
                      'reference_setup_and_solve_s': 11.07},
            'forms': forms,
            'gpu_launches': int(launches),
            'clocks': clk.summary(),
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == '__main__':
    main()
