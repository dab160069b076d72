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
