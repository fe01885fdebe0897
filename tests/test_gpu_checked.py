"""The bounds-checked library, libmlgi_checked.so (built with -DMLGI_CHECKS).

Its kernels check the indices they compute against the extents of the buffers they address; an
index outside is recorded (source line and value) and replaced by 0, so that the access stays in
the buffer, and mlgi_check_device_status reports MLGI_EBOUNDS. Here:
  * the recording and reporting work: the self-test reads through a checked index outside its
    array (redirected to element 0, so nothing leaves the array) and is reported;
  * the normal library refuses that self-test without launching anything;
  * the parity suites of the kernels -- VPLs, ISM splat, pull-push in both forms, final gathering,
    batches, device scene generation, clustered culling, post passes, the bounded wait -- pass under
    the checked library on their small cases, with no violation recorded after any test.
The checked cases run in child processes with MLGI_CHECKED=1, so this process keeps the normal
library.
"""
import os
import re
import subprocess
import sys

import pytest

import mlgi

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "many-lights-gi_gb300")

SELFTEST = """
import mlgi
L = mlgi.lib()
assert L.mlgi_checks_enabled() == 1
ctx = mlgi.Context(0)
assert L.mlgi_check_index_selftest(ctx.h, 3, 4) == mlgi.OK
ctx.check_device_status()
assert L.mlgi_check_index_selftest(ctx.h, 9, 4) == mlgi.OK
try:
    ctx.check_device_status()
except mlgi.MlgiError as e:
    assert e.status == mlgi.EBOUNDS, e
    assert "index 9 out of range" in str(e) and "mlgi_api" in str(e), e
else:
    raise AssertionError("the violation was not reported")
ctx.check_device_status()  # the record was cleared when it was reported
assert L.mlgi_check_index_selftest(ctx.h, -1, 4) == mlgi.OK
try:
    ctx.check_device_status()
    raise AssertionError("the negative index was not reported")
except mlgi.MlgiError as e:
    assert e.status == mlgi.EBOUNDS, e
ctx.close()
print("selftest ok")
"""

CHECKED_SUITES = ["tests/test_gpu_parity.py", "tests/test_gpu_batch.py", "tests/test_gpu_scene.py",
                  "tests/test_gpu_cluster.py", "tests/test_gpu_post.py", "tests/test_gpu_timeout.py"]


def _child(args, timeout):
    env = dict(os.environ, MLGI_CHECKED="1", PYTHONPATH=os.pathsep.join([ROOT, PKG, os.environ.get("PYTHONPATH", "")]))
    return subprocess.run([sys.executable] + args, cwd=ROOT, env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                          text=True, timeout=timeout)


def test_checked_selftest_records_and_reports_an_index_outside_its_array():
    r = _child(["-c", SELFTEST], 300)
    assert r.returncode == 0 and "selftest ok" in r.stdout, r.stdout[-4000:]


def test_normal_library_refuses_the_out_of_range_selftest():
    L = mlgi.lib()
    assert L.mlgi_checks_enabled() == 0
    ctx = mlgi.Context(0)
    assert L.mlgi_check_index_selftest(ctx.h, 9, 4) == mlgi.EINVAL
    assert L.mlgi_check_index_selftest(ctx.h, 3, 4) == mlgi.OK
    assert L.mlgi_check_index_selftest(ctx.h, 0, 0) == mlgi.EINVAL
    ctx.check_device_status()
    ctx.close()


def test_kernel_parity_suites_pass_under_the_checked_library():
    r = _child(["-m", "pytest", "-q", "-x", "-m", "gpu", "-p", "no:cacheprovider"] + CHECKED_SUITES, 1500)
    tail = r.stdout[-6000:]
    assert r.returncode == 0, tail
    m = re.search(r"(\d+) passed", tail)
    assert m and int(m.group(1)) >= 60, tail  # every case of those suites ran
