"""The bench's reference arm (the reference's CPU path, the FP64 oracle port
timed on the host cores) prints the JSON line the harness reads: the same
metric and unit as the GPU arm, impl "reference", an e2e object with no host
copies and a cpu_baseline describing the run.  CPU only."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, 'bench.py'), '--impl', 'reference', '--steps', '1',
                        '--warmup', '0'], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith('{')]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    assert d['impl'] == 'reference'
    assert d['metric'] == 'NSST dec+thresh+rec images/s at 512^2 fp32, batched'
    assert d['unit'] == 'images/s' and d['higher_is_better'] is True
    assert d['value'] > 0 and d['steps'] == 1 and d['n_gpus'] == 1
    assert d['e2e']['value'] == d['value'] and d['e2e']['unit'] == d['unit']
    assert d['e2e']['h2d_bytes_per_step'] == 0 and d['e2e']['d2h_bytes_per_step'] == 0
    cb = d['cpu_baseline']
    assert cb['kind'] in ('port', 'reference') and cb['cores'] >= 1 and cb['sample']
    assert cb['value'] == d['value']
