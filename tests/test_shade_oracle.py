"""CPU: the FP64 reference gradient of the oracle (forward-mode dual numbers) agrees with central
finite differences (h = 1e-4) of the FP64 loss, for both falloffs."""
import numpy as np
import pytest

import oracle
import shade_scene


# With per-pixel random normals some pixels see a light at a grazing angle, where the reference BRDF's
# specular term NDF*G / (4*NdotV*NdotL + 1e-4) varies on a 1e-5 scale in NdotL; a +-1e-4 step in the
# light position cannot resolve it (median error ~5e-4, worst light ~2e-2), a 1e-6 step can (< 1e-6).
# The reference falloff 1 - min(d/r, 1)^1.5 also has a derivative jump at d = r.  So: the specified
# h = 1e-4 is checked on the median over lights, h = 1e-6 on every light.
@pytest.mark.parametrize("falloff,h,tol,stat", [(1, 1e-4, 2e-3, "median"), (1, 1e-6, 1e-5, "max"),
                                                (0, 1e-6, 1e-5, "max")])
def test_dual_gradient_matches_central_differences(falloff, h, tol, stat):
    s = shade_scene.make(160, 96, 64, seed=11)
    g7 = oracle.cs_shade_grad_f64(s["view"], s["W"], s["H"], shade_scene.gb(s), shade_scene.lists(s), s["pos"],
                                  s["lights"], s["L"], s["grad"], falloff=falloff)
    active = np.nonzero(np.abs(g7).sum(1) > 0)[0]
    assert len(active) >= 8, "the scene must give most lights a non-zero gradient"
    errs = []
    for l in active[:12]:
        theta = np.array([*s["pos"][4 * l:4 * l + 3], *s["lights"][4 * l:4 * l + 4]], np.float64)
        fd = np.zeros(7)
        for t in range(7):
            tp, tm = theta.copy(), theta.copy()
            tp[t] += h
            tm[t] -= h
            fd[t] = (oracle.cs_shade_light_loss_f64(s["view"], s["W"], s["H"], shade_scene.gb(s), shade_scene.lists(s),
                                                    int(l), tp, s["grad"], falloff) -
                     oracle.cs_shade_light_loss_f64(s["view"], s["W"], s["H"], shade_scene.gb(s), shade_scene.lists(s),
                                                    int(l), tm, s["grad"], falloff)) / (2 * h)
        errs.append(np.linalg.norm(fd - g7[l]) / max(np.linalg.norm(g7[l]), 1e-12))
    assert len(errs) >= 8
    value = float(np.median(errs)) if stat == "median" else float(np.max(errs))
    assert value < tol, (stat, value, errs)


def test_forward_radiance_is_consistent_with_gradient_linearity():
    """Loss = <grad, radiance> is linear in the light colour: dLoss/dcolour * colour summed over the
    three channels reproduces each light's share of the loss."""
    s = shade_scene.make(96, 64, 24, seed=3)
    g7 = oracle.cs_shade_grad_f64(s["view"], s["W"], s["H"], shade_scene.gb(s), shade_scene.lists(s), s["pos"],
                                  s["lights"], s["L"], s["grad"], falloff=1)
    for l in range(s["L"]):
        theta = np.array([*s["pos"][4 * l:4 * l + 3], *s["lights"][4 * l:4 * l + 4]], np.float64)
        share = oracle.cs_shade_light_loss_f64(s["view"], s["W"], s["H"], shade_scene.gb(s), shade_scene.lists(s), l,
                                               theta, s["grad"], 1)
        assert abs(share - float(np.dot(g7[l, 3:6], theta[3:6]))) <= 1e-9 * max(1.0, abs(share))
