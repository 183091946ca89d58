"""bench.py's reference arm: the oracle on the host cores, with inputs built by the oracle alone.

The arm must load no product code (its timed region and its inputs), and print the same
workload `config` as the GPU arm.
"""
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import sys
sys.path.insert(0, %r)
import bench
from minisod2d_gb300 import workload
cfg = workload.custom(4, 3, 0.05)
host = bench.OracleHostCase(cfg)
geom, ne, mu = bench.cpu_sample_case(cfg, host, 8)
bench.cpu_step(cfg, host, geom, ne, mu, 2)
print(bench.workload_config(cfg, host.nelem, host.npoin))
maps = open("/proc/self/maps").read()
print("PRODUCT_LOADED" if "libmsod.so" in maps else "PRODUCT_NOT_LOADED")
print("ORACLE_LOADED" if "libmsod_oracle.so" in maps else "ORACLE_NOT_LOADED")
""" % ROOT


def test_reference_arm_loads_no_product_library():
    out = subprocess.run([sys.executable, "-c", SCRIPT], capture_output=True, text=True, cwd=ROOT, timeout=300)
    assert out.returncode == 0, out.stderr
    assert "PRODUCT_NOT_LOADED" in out.stdout
    assert "ORACLE_LOADED" in out.stdout
    assert "'workload': 'custom_p4_n3'" in out.stdout
