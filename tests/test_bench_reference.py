"""The benchmark's reference arm (the oracle port of the reference's
traversal on the host cores) runs without a GPU and without the GPU library:
it builds its scene with the oracle's own generator, so no libvt.so is
mapped into its process, and it prints the contract's JSON line."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent

PROBE = """
import runpy, sys
sys.argv = ['bench.py', '--impl', 'reference', '--steps', '10', '--warmup', '0']
runpy.run_path('bench.py', run_name='__main__')
maps = open('/proc/self/maps').read()
print('MAPPED', 'libvt.so' in maps, 'liboracle.so' in maps)
"""


def test_reference_arm_loads_only_the_oracle():
    out = subprocess.run([sys.executable, "-c", PROBE], cwd=ROOT, capture_output=True, text=True, timeout=600,
                         check=True).stdout.splitlines()
    line = json.loads(next(s for s in out if s.startswith("{")))
    assert line["impl"] == "reference" and line["metric"] == "Grays/s" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0
    assert out[-1] == "MAPPED False True"
