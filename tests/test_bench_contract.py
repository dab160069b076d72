"""bench.py's JSON contract, on CPU: the reference arm (the C oracle timed on
the host's cores) prints exactly one JSON line with every key the contract
names, its e2e block carrying zero host<->device bytes."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    env = dict(os.environ)
    out = subprocess.run([sys.executable, os.path.join(ROOT, 'bench.py'), '--impl', 'reference', '--steps', '1',
                          '--warmup', '1'], cwd=ROOT, env=env, capture_output=True, text=True, timeout=900)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith('{')]
    assert len(lines) == 1, out.stdout[-2000:]
    d = json.loads(lines[0])
    for k in ('metric', 'value', 'unit', 'n_gpus', 'steps', 'warmup', 'ms_per_step', 'higher_is_better', 'scaling',
              'vs_baseline', 'dtype', 'data', 'config', 'impl', 'cpu_baseline', 'e2e'):
        assert k in d, k
    assert d['impl'] == 'reference' and d['n_gpus'] == 1 and d['steps'] == 1 and d['warmup'] == 1
    assert d['value'] > 0 and d['unit'] == 'solves/s' and d['higher_is_better'] is True
    assert 'workload' in d['config'] and d['config']['vcycles'] == 10 and d['config']['final_rel'] <= 1e-10
    cb = d['cpu_baseline']
    assert set(cb) >= {'value', 'unit', 'cores', 'kind', 'sample'} and cb['value'] == d['value'] and cb['cores'] >= 1
    assert d['e2e'] == {'value': d['value'], 'unit': d['unit'], 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}


import pytest


@pytest.mark.gpu
def test_native_line():
    """The GPU arm (plain FP64 path only): roofline, cpu_baseline, e2e with
    the bytes actually copied, launch count and clocks."""
    out = subprocess.run([sys.executable, os.path.join(ROOT, 'bench.py'), '--steps', '3', '--warmup', '3',
                          '--no-forms', '--cpu-budget', '2'], cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith('{')]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d['value'] > 0 and d['dtype'] == 'f64' and d['n_gpus'] == 1 and d['config']['final_rel'] <= 1e-10
    r = d['roofline']
    assert r['bound'] == 'hbm' and r['unit'] == 'GB/s' and 0 < r['frac'] < 1.5
    assert abs(r['frac'] - r['achieved'] / r['peak']) < 1e-9 and r['traffic'] and r['traffic'] > 0
    assert 0 < r['fp64_pipe']['frac'] < 1.5
    assert r['avg_launch_us'] > 0 and r['eager_avg_launch_us'] > 0 and 'graph' in r['timing']
    e = d['e2e']
    assert e['unit'] == 'solves/s' and e['h2d_bytes_per_step'] > 0 and e['d2h_bytes_per_step'] > 0
    assert d['gpu_launches'] > 1000
    assert d['cpu_baseline']['kind'] == 'port' and d['cpu_baseline']['value'] > 0
    assert {'sm_mhz', 'sm_max_mhz', 'reasons'} <= set(d['clocks'])
    s = d['setup']
    assert 0 < s['host_build_s'] < s['setup_and_solve_s'] and s['first_solve_s'] > 0
    pk = d['config']['per_kernel']
    assert pk['relax']['launches_per_cycle'] > 0 and pk['relax']['achieved_gbs'] > 0
    assert 0 < pk['coarse_load']['frac'] < 1.5 and pk['ghost']['achieved_gbs'] is None


@pytest.mark.gpu
def test_eager_vcycle_mode():
    """The profiling aid: one eager V-cycle between cudaProfilerStart/Stop."""
    out = subprocess.run([sys.executable, os.path.join(ROOT, 'bench.py'), '--eager-vcycle'], cwd=ROOT,
                         capture_output=True, text=True, timeout=900)
    assert out.returncode == 0, out.stderr[-2000:]
    d = json.loads([l for l in out.stdout.splitlines() if l.startswith('{')][0])
    assert d['eager_vcycle'] == 'done' and d['levels'] == 7 and d['kernels'] > 50
    assert d['precision'] == 'fp64' and d['relax_forms'][0] == 1


def test_clock_summary_keeps_the_timed_region():
    """The clock record of the bench line comes from the samples taken
    between the timed region's start and end marks; throttle reasons are read
    from those samples only."""
    sys.path.insert(0, ROOT)
    import bench
    c = bench.ClockSampler()
    row = lambda mhz, hw: [str(mhz), '2070', '900.0', 'Active' if hw else 'Not Active', 'Not Active',
                           'Not Active', 'Not Active']
    c.rows = [(0.0, row(1000, True)), (1.0, row(2070, False)), (1.1, row(2060, False)), (5.0, row(500, True))]
    c.t0, c.t1 = 0.9, 1.2
    s = c.summary()
    assert s['samples'] == 2 and s['in_region'] and s['sm_mhz'] == 2065.0 and s['reasons'] == []
    c.t0, c.t1 = 10.0, 11.0             # nothing inside: every sample, flagged
    s = c.summary()
    assert s['samples'] == 4 and not s['in_region'] and s['reasons'] == ['hw_slowdown']
