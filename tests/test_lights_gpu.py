"""GPU: the point-light bouncer (vren_demo's bounce_point_lights.comp) against the CPU restatement,
bit for bit: lights inside and outside the box (clamped onto a face), zero and negative direction
components, many bounces (more than the 32-iteration cap), no travel, large light counts."""
import numpy as np
import pytest
import torch

import oracle
import vren_gb300 as vg
import vren_gb300.clustered_shading as cs

pytestmark = pytest.mark.gpu


def same_bits(a, b):
    """Bit-identical, except that NaNs compare as NaN: a light with a zero direction divides 0/0,
    and the NaN payload (0x7fffffff on the GPU, 0x7fc00000 on x86/Arm) is unspecified in GLSL."""
    a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
    na, nb = np.isnan(a), np.isnan(b)
    return np.array_equal(na, nb) and np.array_equal(a[~na].view(np.uint32), b[~nb].view(np.uint32))


def run(device, pos, dirs, L, lo, hi, speed, dt):
    p = torch.from_numpy(np.ascontiguousarray(pos, np.float32).reshape(-1)).to(device)
    d = torch.from_numpy(np.ascontiguousarray(dirs, np.float32).reshape(-1)).to(device)
    cs.bounce_point_lights(None, p, d, L, lo, hi, speed, dt)
    torch.cuda.synchronize()
    return p.cpu().numpy(), d.cpu().numpy()


@pytest.mark.parametrize("L", [1, 7, 1000, 65537, 1 << 20])
@pytest.mark.parametrize("speed,dt", [(3.0, 0.016), (3.0, 4.0), (50.0, 10.0), (0.0, 1.0), (2.0, -1.0)])
def test_bounce_matches_oracle(cuda, L, speed, dt):
    rng = np.random.default_rng([L, int(speed * 100), int(dt * 1000) + 1000])
    pos = np.zeros((L, 4), np.float32)
    pos[:, :3] = rng.uniform(-14, 14, (L, 3))
    pos[:, 2] += 15
    pos[:, 3] = 1
    dirs = np.zeros((L, 4), np.float32)
    dirs[:, :3] = rng.standard_normal((L, 3))
    dirs[::5, 0] = 0.0          # moving parallel to a pair of faces
    dirs[::7, 1] = -0.0
    dirs[::11, :3] = 0.0        # not moving at all
    lo, hi = [-10.0, -5.0, 0.0], [10.0, 5.0, 30.0]
    gp, gd = run(cuda, pos, dirs, L, lo, hi, speed, dt)
    ep, ed = oracle.bounce_point_lights(pos, dirs, L, lo, hi, speed, dt)
    assert same_bits(gp, ep)
    assert same_bits(gd, ed)
    assert vg.device_error() == 0


def test_bounce_repeated_frames_stay_in_box(cuda):
    """Lights that start inside the box stay inside over many frames (the demo's use), GPU = CPU."""
    L = 4096
    rng = np.random.default_rng(3)
    lo, hi = np.array([-10.0, -5.0, 0.0], np.float32), np.array([10.0, 5.0, 30.0], np.float32)
    pos = np.zeros((L, 4), np.float32)
    pos[:, :3] = rng.uniform(lo, hi, (L, 3))
    dirs = np.zeros((L, 4), np.float32)
    dirs[:, :3] = rng.standard_normal((L, 3))
    p = torch.from_numpy(pos.reshape(-1).copy()).to(cuda)
    d = torch.from_numpy(dirs.reshape(-1).copy()).to(cuda)
    ep, ed = pos.reshape(-1).copy(), dirs.reshape(-1).copy()
    for _ in range(30):
        cs.bounce_point_lights(None, p, d, L, lo, hi, 5.0, 0.25)
        ep, ed = oracle.bounce_point_lights(ep, ed, L, lo, hi, 5.0, 0.25)
    gp = p.cpu().numpy()
    assert same_bits(gp, ep)
    assert np.array_equal(d.cpu().numpy().view(np.uint32), ed.view(np.uint32))
    q = gp.reshape(-1, 4)[:, :3]
    assert np.all(q >= lo - 1e-3) and np.all(q <= hi + 1e-3)


def test_bounce_arguments(cuda):
    p = torch.zeros(8, dtype=torch.float32, device=cuda)
    with pytest.raises(Exception):
        cs.bounce_point_lights(None, p[1:], p, 1, [0, 0, 0], [1, 1, 1], 1.0, 1.0)  # unaligned
    cs.bounce_point_lights(None, p, p, 0, [0, 0, 0], [1, 1, 1], 1.0, 1.0)  # nothing to do
