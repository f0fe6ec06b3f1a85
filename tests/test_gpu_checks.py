"""The checked build (RT_DEVICE_CHECKS=1) on the GPU.

Compute-sanitizer is not available, so a second library,
librt_gb300_checked.so, checks every node, primitive, ray, material and path
index its kernels use and records violations in a per-scene word instead of
faulting.  A subprocess runs ray queries (both node layouts, sorted, any-hit,
Moller-Trumbore, deep stacks, host buffers) and wavefront renders (two pixel
chunks on two streams) through it; every check word must stay clear and
every result must equal the normal build's.
"""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent

SCRIPT = r'''
import sys, numpy as np, torch
sys.path.insert(0, sys.argv[1])
import raytracergpu_mastersproject_gb300 as rt
from raytracergpu_mastersproject_gb300 import workloads as W
out = {"compiled": np.array([rt.device_checks_compiled()])}
checks = []

def dev(sc, rays, **kw):
    d_r = torch.from_numpy(rays.view(np.uint8)).cuda()
    d_h = torch.empty(len(rays) * 8, dtype=torch.uint8, device="cuda")
    sc.trace(d_r, d_h, **kw)
    torch.cuda.synchronize()
    return d_h.cpu().numpy().view(np.uint64)

tris3, rays3 = W.config3(200_000, 300_000)
for w in (2, 4):
    with rt.Scene(tris3, node_width=w) as sc:
        out[f"soup{w}"] = dev(sc, rays3)
        out[f"soup{w}_sort"] = dev(sc, rays3, sort=True)
        out[f"soup{w}_any"] = dev(sc, rays3, any_hit=True)
        out[f"soup{w}_mt"] = dev(sc, rays3, mt=True)
        out[f"soup{w}_host"] = sc.trace_host(rays3).view(np.uint64)
        checks.append(sc.device_checks())
t1, ubo1, r1 = rt.gen_config1()
with rt.Scene(t1, bvh_mode=rt.BVH_REFERENCE) as sc:
    out["config1_ref"] = dev(sc, r1)
    checks.append(sc.device_checks())
rng = np.random.default_rng(3)
n = 20_000
dense = np.zeros(n, rt.TRIANGLE_DTYPE)
c = rng.normal(0.0, 0.05, (n, 3)).astype(np.float32)
for k in ("v0", "v1", "v2"):
    dense[k][:, :3] = c + rng.normal(0.0, 0.5, (n, 3)).astype(np.float32)
with rt.Scene(dense) as sc:
    out["dense"] = dev(sc, rays3[:50_000])
    checks.append(sc.device_checks())
tris2, mats2 = rt.gen_spheres_scene(2, 64, 3, 0.05)
ubo2 = rt.make_ubo((0.0, 3.0, 28.0), (0.0, 0.0, 0.0), fov=40.0, depth=8, random_state=2,
                   num_triangles=len(tris2), num_materials=len(mats2))
with rt.Scene(tris2, materials=mats2) as sc:
    # 320 x 240 x 4 samples: the frame runs as two pixel chunks on two streams
    acc = torch.empty(320 * 240 * 4, dtype=torch.float32, device="cuda")
    for mode in (rt.SHADE_EXTENDED, rt.SHADE_REFERENCE):
        rt.accum_clear(acc, 320, 240)
        sc.render(ubo2, acc, 320, 240, 4, shade_mode=mode, background=(0.6, 0.7, 1.0))
        torch.cuda.synchronize()
        out[f"render{mode}"] = acc.cpu().numpy()
    checks.append(sc.device_checks())
out["checks"] = np.array(checks, dtype=np.uint64)
np.savez(sys.argv[2], **out)
'''


def test_checked_build_is_clean_and_equal(tmp_path):
    from raytracergpu_mastersproject_gb300 import _build

    checked = _build.build(checked=True)
    script = tmp_path / "run.py"
    script.write_text(SCRIPT)
    env_checked = dict(os.environ, RT_GB300_LIB=str(checked))
    r = subprocess.run([sys.executable, str(script), str(ROOT), str(tmp_path / "checked.npz")], env=env_checked,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    normal = dict(os.environ)
    normal.pop("RT_GB300_LIB", None)
    r = subprocess.run([sys.executable, str(script), str(ROOT), str(tmp_path / "normal.npz")], env=normal,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    a = np.load(tmp_path / "checked.npz")
    b = np.load(tmp_path / "normal.npz")
    assert a["compiled"][0] == 1 and b["compiled"][0] == 0
    assert np.all(a["checks"] == 0), a["checks"]
    for k in a.files:
        if k not in ("compiled", "checks"):
            assert np.array_equal(a[k], b[k]), k
