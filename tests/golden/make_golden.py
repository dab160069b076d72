"""Extract the reference's recorded outputs into tests/golden/reference_outputs.json.

Usage: python make_golden.py <path of the reference repository>.  The
reference is MATLAB and cannot run here; its own verification run (MATLAB R2026a) recorded these numbers in
verification/, and they are the golden values the oracle is pinned to.
"""
import csv
import json
import os
import re
import sys

if len(sys.argv) != 2:
    sys.exit('usage: make_golden.py <path of the reference repository>')
REF = sys.argv[1]
VER = os.path.join(REF, 'verification')
out = {}

# G1: starfish residual history (verification/starfish-full-residual.csv)
with open(os.path.join(VER, 'starfish-full-residual.csv')) as f:
    rows = list(csv.DictReader(f))
out['starfish_residual_history'] = [float(r['absoluteResidual']) for r in rows]

# G2: starfish summary (verification/starfish-full.json)
with open(os.path.join(VER, 'starfish-full.json')) as f:
    sj = json.load(f)
out['starfish'] = {k: sj[k] for k in ('baseCells', 'levels', 'epsilon', 'boundaryPoints', 'visibleCells',
                                      'storedAmrCells', 'vcycles', 'relativeResidual', 'balanceDefect',
                                      'patchesPerLevel', 'cellsPerLevel', 'interfaceBandCells',
                                      'uncoveredBandCells', 'setupAndSolveSeconds', 'uniformSetupAndSolveSeconds',
                                      'uniformRelativeResiduals')}

# G3/G4: README examples (verification/readme-examples.txt)
stage_re = re.compile(r'\[ebsam\] stage (\d+): (\d+) AMR level\(s\), (\d+) V-cycle\(s\), \|r\|/\|f\| = ([0-9.e+-]+), '
                      r'avg factor ([0-9.]+), (\d+) visible cells')
added_re = re.compile(r'\[(ebsam|ebtsam)\] added level (\d+) \((\d+) patch\(es\), (\d+) cells, h = ([0-9.e+-]+)\)')
heat_re = re.compile(r'\[ebsam-p\] step\s+(\d+)/(\d+)\s+t=([0-9.]+)\s+V=(\d+)\s+rel=([0-9.e+-]+)\s+levels=(\d+)\s+'
                     r'cells=(\d+)\s+mass=([0-9.e+-]+)')
stages, added, heat = [], [], []
with open(os.path.join(VER, 'readme-examples.txt')) as f:
    for line in f:
        m = stage_re.search(line)
        if m:
            stages.append({'stage': int(m[1]), 'amrLevels': int(m[2]), 'vcycles': int(m[3]), 'rel': m[4],
                           'avgFactor': m[5], 'visibleCells': int(m[6])})
        m = added_re.search(line)
        if m:
            added.append({'tree': m[1] == 'ebtsam', 'level': int(m[2]), 'np': int(m[3]), 'cells': int(m[4]),
                          'h': m[5]})
        m = heat_re.search(line)
        if m:
            heat.append({'step': int(m[1]), 'nsteps': int(m[2]), 't': float(m[3]), 'V': int(m[4]), 'rel': m[5],
                         'levels': int(m[6]), 'cells': int(m[7]), 'mass': m[8]})
out['readme_ring_stages'] = stages[:3]
out['readme_tree_stages'] = stages[3:6]
out['readme_ring_added'] = [a for a in added if not a['tree']]
out['readme_tree_added'] = [a for a in added if a['tree']]
out['readme_heat_steps'] = heat

# G5: suite output lines used by the tests (verification/suite-output.txt)
suite = open(os.path.join(VER, 'suite-output.txt')).read().splitlines()
t1 = []
for line in suite:
    m = re.match(r'\s+m=\s*(\d+)\s+err_inf=([0-9.e+-]+)\s+err_l2=([0-9.e+-]+)\s+factor=([0-9.]+)\s+V=(\d+)\s+t=', line)
    if m:
        t1.append({'m': int(m[1]), 'err_inf': m[2], 'err_l2': m[3], 'factor': m[4], 'V': int(m[5])})
out['suite_T1_uniform_mms'] = t1[:4]
t3 = []
for line in suite:
    m = re.match(r'\s+\[(qif|lif)\] m0=\s*(\d+) L=(\d): err=([0-9.e+-]+) factor=([0-9.]+) mass=([0-9.e+-]+) V=(\d+)',
                 line)
    if m:
        t3.append({'interp': m[1], 'm0': int(m[2]), 'L': int(m[3]), 'err': m[4], 'factor': m[5], 'mass': m[6],
                   'V': int(m[7])})
out['suite_T3_box_in_box'] = t3[:24]        # EllipticBSAM/tests/runAllTests.m
out['suite_T3_box_in_box_tree'] = t3[24:48]  # EllipticBSAMTree/tests/runAllTreeTests.m


def section(name, which):
    """Lines of suite section `name` (e.g. 'T2'), occurrence `which` (0: the
    QC-ring suite, 1: the tree suite)."""
    starts = [i for i, l in enumerate(suite) if l.startswith('=== ' + name + ':')]
    i = starts[which] + 1
    lines = []
    while i < len(suite) and not suite[i].startswith('===') and suite[i].strip():
        lines.append(suite[i])
        i += 1
    return lines


for which, tag in ((0, ''), (1, '_tree')):
    t2 = []
    for line in section('T2', which):
        m = re.match(r'\s+m=\s*(\d+)\s+err_inf=([0-9.e+-]+)\s+err_l2=([0-9.e+-]+)\s+factor=([0-9.]+)\s+V=(\d+)', line)
        if m:
            t2.append({'m': int(m[1]), 'err_inf': m[2], 'err_l2': m[3], 'factor': m[4], 'V': int(m[5])})
    out['suite_T2_pure_neumann' + tag] = t2
    t4 = []
    for line in section('T4', which):
        m = re.match(r'\s+m0=\s*(\d+)\s+err_inf=([0-9.e+-]+)\s+factor=([0-9.]+)\s+level-2 patches=(\d+)\s+mass=([0-9.e+-]+)',
                     line)
        if m:
            t4.append({'m0': int(m[1]), 'err_inf': m[2], 'factor': m[3], 'np2': int(m[4]), 'mass': m[5]})
    out['suite_T4_lshape' + tag] = t4
    t5 = []
    for line in section('T5', which):
        m = re.match(r'\s+MaxLevels=(\d) \(got (\d)\): err_inf=([0-9.e+-]+)\s+err_l2=([0-9.e+-]+)\s+factor=([0-9.]+)'
                     r'\s+dof=(\d+)', line)
        if m:
            t5.append({'MaxLevels': int(m[1]), 'got': int(m[2]), 'err_inf': m[3], 'err_l2': m[4], 'factor': m[5],
                       'dof': int(m[6])})
    out['suite_T5_adaptive' + tag] = t5
    t7 = []
    for line in section('T7', which):
        m = re.match(r'\s+levels=(\d)\s+corrections=(\d) : mass defect \(rel\) = ([0-9.e+-]+)\s+err=([0-9.e+-]+)', line)
        if m:
            t7.append({'levels': int(m[1]), 'corrections': int(m[2]), 'mass': m[3], 'err': m[4]})
    out['suite_T7_mass' + tag] = t7
    t8 = []
    for line in section('T8', which):
        m = re.match(r'\s+patches=(\d+)\s+min width=(\d+) \(fine cells\)\s+factor=([0-9.]+)\s+err=([0-9.e+-]+)'
                     r'\s+mass=([0-9.e+-]+)', line)
        if m:
            t8.append({'patches': int(m[1]), 'minw': int(m[2]), 'factor': m[3], 'err': m[4], 'mass': m[5]})
    out['suite_T8_scattered' + tag] = t8
# T9 (EllipticBSAMTree/tests/runAllTreeTests.m:242-283): tree invariants and
# the straddling-feature scenario; T6 (runAllTests.m:148-155): the 2-level
# QIF factors of T3 for m0 = 32..256.
t9 = {}
for line in section('T9', 0):
    m = re.match(r'\s+T5 hierarchy: (\d+) AMR level\(s\), per-level patches \[([^\]]+)\], max children (\d+)', line)
    if m:
        t9.update({'depth': int(m[1]), 'per_level': [int(v) for v in m[2].split()], 'max_children': int(m[3])})
    m = re.match(r'\s+straddle scenario: level-2 patches=(\d+), level-3 patches=(\d+), parents=\[([^\]]+)\]', line)
    if m:
        t9.update({'np2': int(m[1]), 'np3': int(m[2]), 'parents': [int(v) for v in m[3].split()]})
    m = re.match(r'\s+solver: V=(\d+) rel=([0-9.e+-]+) factor=([0-9.]+) mass=([0-9.e+-]+) err=([0-9.e+-]+)', line)
    if m:
        t9.update({'V': int(m[1]), 'rel': m[2], 'factor': m[3], 'mass': m[4], 'err': m[5]})
out['suite_T9_tree'] = t9
for which, tag in ((0, ''), (1, '_tree')):
    t6 = {}
    for line in section('T6', which):
        m = re.match(r'\s+m0 = \[([^\]]+)\]', line)
        if m:
            t6['m0'] = [int(v) for v in m[1].split()]
        m = re.match(r'\s+factors = \[([^\]]+)\]', line)
        if m:
            t6['factors'] = m[1].split()
    out['suite_T6_h_independence' + tag] = t6
# Diffuse-domain suite (DiffuseDomainBSAM/tests/runDdTests.m): D1 star /
# Neumann (uniform, adaptive, adaptive without corrections) and D2 disc /
# Dirichlet penalty.
d1 = []
for line in section('D1', 0):
    m = re.match(r'\s+eps=([0-9.]+)\s+uni\(L2\)=([0-9.e+-]+)\s+amr\(L2\)=([0-9.e+-]+)\s+noCorr\(L2\)=([0-9.e+-]+)'
                 r'\s+\| mass: ([0-9.e+-]+) / ([0-9.e+-]+) / ([0-9.e+-]+) \| amr factor ([0-9.]+)', line)
    if m:
        d1.append({'eps': float(m[1]), 'uni_l2': m[2], 'amr_l2': m[3], 'nocorr_l2': m[4], 'mass_uni': m[5],
                   'mass_amr': m[6], 'mass_nocorr': m[7], 'amr_factor': m[8]})
for line in section('D3', 0):           # cells(uni) / cells(amr) = the D1 solves' dof
    m = re.match(r'\s+([0-9.]+)\s+(\d+)\s+(\d+)\s+[0-9.]+x', line)
    if m:
        for row in d1:
            if row['eps'] == float(m[1]):
                row.update({'dof_uni': int(m[2]), 'dof_amr': int(m[3])})
out['suite_D1_star_neumann'] = d1
d1b = []
for line in section('D1b', 0):
    m = re.match(r'\s+eps=([0-9.]+)\s+E\(eps/h=12.8\)=([0-9.e+-]+)\s+E\(25.6\)=([0-9.e+-]+)\s+h-rate=(-?[0-9.]+)'
                 r'\s+model M=([0-9.e+-]+)', line)
    if m:
        d1b.append({'eps': float(m[1]), 'E1': m[2], 'E2': m[3], 'h_rate': m[4], 'M': m[5]})
out['suite_D1b_circle_model_error'] = d1b
d2 = []
for line in section('D2', 0):
    m = re.match(r'\s+eps=([0-9.]+)\s+L2=([0-9.e+-]+)\s+Linf=([0-9.e+-]+)\s+factor=([0-9.]+)\s+dof=(\d+)', line)
    if m:
        d2.append({'eps': float(m[1]), 'l2': m[2], 'linf': m[3], 'factor': m[4], 'dof': int(m[5])})
out['suite_D2_disc_dirichlet'] = d2
# Parabolic suite (ParabolicBSAM/tests/runParabolicTests.m P1-P4) and its
# regressions (runParabolicRegressions.m, the 'PASS CN' lines).
par = {'P1a': {}, 'P1b': [], 'P2_steps': [], 'CN_mass': []}
for line in section('P1', 0):
    m = re.match(r'\s+(be|bdf2|cn)\s+Cauchy diffs \[([^\]]+)\]', line)
    if m:
        par['P1a'][m[1]] = m[2].split()
    m = re.match(r'\s+bdf2\s+h=1/(\d+)\s+Dt=([0-9.]+)\s+err_inf=([0-9.e+-]+)\s+<V>=([0-9.]+)\s+regrids=(\d+)', line)
    if m:
        par['P1b'].append({'h_inv': int(m[1]), 'Dt': float(m[2]), 'err_inf': m[3], 'meanV': m[4],
                           'regrids': int(m[5])})
for line in section('P2', 0):
    m = heat_re.search(line)
    if m:
        par['P2_steps'].append({'step': int(m[1]), 'V': int(m[4]), 'rel': m[5], 'levels': int(m[6]),
                                'cells': int(m[7]), 'mass': m[8]})
    m = re.match(r'\s+steps=(\d+)\s+regrids=(\d+)\s+<V/step>=([0-9.]+)\s+mass drift=([0-9.e+-]+) \(mass=([0-9.]+)\)',
                 line)
    if m:
        par['P2'] = {'steps': int(m[1]), 'regrids': int(m[2]), 'meanV': m[3], 'drift': m[4], 'mass': m[5]}
    m = re.match(r'\s+final levels: (\d+)', line)
    if m:
        par['P2']['final_levels'] = int(m[1])
for line in section('P3', 0):
    m = re.search(r'finest level covers it: (\d)', line)
    if m:
        par['P3'] = {'covered': int(m[1])}
    m = re.match(r'\s+cells=(\d+) .*regrids=(\d+), <V>=([0-9.]+)', line)
    if m:
        par['P3'].update({'cells': int(m[1]), 'regrids': int(m[2]), 'meanV': m[3]})
for line in section('P4', 0):
    m = re.match(r'\s+P2 mean V-cycles/step: ([0-9.]+)', line)
    if m:
        par['P4'] = {'meanV': m[1]}
    m = re.search(r'max\|u\| = ([0-9.]+)', line)
    if m:
        par['P4']['umax_big_dt'] = m[1]
for line in suite:
    m = re.match(r'PASS CN time-dependent C: errors \[([^\]]+)\]', line)
    if m:
        par['CN_reaction_errors'] = m[1].split()
    m = re.match(r'PASS CN time-dependent D/BC: Cauchy \[([^\]]+)\]', line)
    if m:
        par['CN_diffusion_cauchy'] = m[1].split()
    m = re.match(r'PASS CN composite mass: regrid=(\d) drift=([0-9.e+-]+) rel=([0-9.e+-]+)', line)
    if m:
        par['CN_mass'].append({'regrid': int(m[1]), 'drift': m[2], 'rel': m[3]})
out['suite_parabolic'] = par
out['source'] = {'repository': 'BSAM-in-MATLAB', 'files': ['verification/starfish-full-residual.csv',
                                                          'verification/starfish-full.json',
                                                          'verification/readme-examples.txt',
                                                          'verification/suite-output.txt'],
                 'matlab': sj.get('matlab')}
dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'reference_outputs.json')
with open(dst, 'w') as f:
    json.dump(out, f, indent=1)
print('wrote', dst)
