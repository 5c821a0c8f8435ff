"""bench.py's launch logic and its CPU legs, on the CPU.

* The reference arm (`--impl reference`, the CPU restatement of merian's `pt`) builds its scene and
  camera from the oracle library alone: the process never maps the package's CUDA library.
* `--gpus N` outside torchrun starts N ranks (rank 0 reports `n_gpus` = N); under torchrun a
  `--gpus` that disagrees with WORLD_SIZE is refused.
* The oracle's scene generators and camera basis give the package library's bits.
"""
import json
import os
import subprocess
import sys

import numpy as np

from conftest import ROOT

SMALL = ["--workload", "cornell-256-16spp", "--steps", "1", "--warmup", "0",
         "--cpu-seconds", "0.1"]


def _json_line(out: str) -> dict:
    lines = [ln for ln in out.splitlines() if ln.startswith("{")]
    assert lines, out
    return json.loads(lines[-1])


def test_reference_arm_maps_no_package_library():
    code = (
        "import runpy, sys\n"
        f"sys.argv = ['bench.py', '--impl', 'reference', *{SMALL!r}]\n"
        "runpy.run_path('bench.py', run_name='__main__')\n"
        "maps = open('/proc/self/maps').read()\n"
        "print('MAPS', 'libgbpt' in maps, 'liboracle' in maps)\n")
    env = dict(os.environ)
    env.pop("WORLD_SIZE", None)
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True,
                       env=env, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    line = _json_line(r.stdout)
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["cores"] >= 1
    assert "MAPS False True" in r.stdout


def test_gpus_flag_starts_that_many_ranks():
    env = dict(os.environ)
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK", "MASTER_ADDR", "MASTER_PORT"):
        env.pop(k, None)
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--gpus", "2", *SMALL],
                       cwd=ROOT, capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = _json_line(r.stdout)
    assert line["n_gpus"] == 2
    # one line: rank 0 reports, the other rank exits without work
    assert sum(ln.startswith("{") for ln in r.stdout.splitlines()) == 1


def test_gpus_flag_must_match_world_size():
    env = dict(os.environ, WORLD_SIZE="3")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--gpus", "2", *SMALL],
                       cwd=ROOT, capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 2
    assert "WORLD_SIZE" in r.stderr


def test_oracle_generators_and_camera_match_library():
    from merian_gb300 import scene as S
    from oracle import binding as O
    a = S.soup(S.BASE_SEED, 5000, 32, (64, 32))
    b = S.soup(S.BASE_SEED, 5000, 32, (64, 32), lib=O.generator())
    for k in ("vertices", "indices", "geometries", "materials", "env"):
        assert np.array_equal(np.asarray(getattr(a, k)).view(np.uint8),
                              np.asarray(getattr(b, k)).view(np.uint8)), k
    c1 = S.cornell(S.BASE_SEED)
    c2 = S.cornell(S.BASE_SEED, lib=O.generator())
    assert np.array_equal(c1.vertices.view(np.uint8), c2.vertices.view(np.uint8))
    assert np.array_equal(c1.materials.view(np.uint8), c2.materials.view(np.uint8))
    for name in S.WORKLOADS:
        assert bytes(S.workload_camera(name)) == bytes(O.workload_camera(name)), name
    for pos, tgt, fov, asp in [((0.1, 2.0, -3.0), (0.4, -0.2, 0.9), 25.0, 1.0),
                               ((5.0, 5.0, 5.0), (0.0, 0.0, 0.0), 70.0, 2.39)]:
        assert bytes(S.look_at(pos, tgt, (0, 1, 0), fov, asp)) == \
            bytes(O.look_at(pos, tgt, (0, 1, 0), fov, asp))
