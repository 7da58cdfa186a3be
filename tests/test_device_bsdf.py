"""The device principled BSDF on its own (rtx_bsdf_eval / rtx_bsdf_sample,
the code the shading kernel inlines) against the 3,000 golden
PrincipledBSDF::Eval / Sample cases the reference's own sources produced
(src/material.cpp:143-204, 206-295; tests/golden/bsdf.npz): random materials
with metallic 0 / 1 / random, spec_trans 0 / 1 / random (so refraction and
total internal reflection occur), clearcoat on and off, rays from inside and
outside.

Both sides use the same arithmetic in the same order with --fmad=false, so
results agree bit for bit except where a transcendental (sqrtf is exact;
powf, logf, cosf, sinf are not) rounds one ulp apart between the CUDA math
library and the host C library.  Eval calls a transcendental only in its
clearcoat lobe (GTR1's logf) and its refraction lobe (powf of the base
colour), so materials with neither lobe (clearcoat = 0 and spec_trans = 0, or
metallic = 1, which zeroes both weights) must match bit for bit; every other
case must agree within 1e-4 relative.  Sample draws its azimuth through
cosf / sinf in every lobe, so it is held to the same Sample() return value on
every case and 1e-4 on >= 99.5 % of them (a one-ulp change can move a
direction across a total-internal-reflection boundary or a lobe choice).  The
counts of cases that differ are printed.
"""
import numpy as np
import pytest

from helpers import bits, rel_close

pytestmark = pytest.mark.gpu


def _classes(g):
    m = g["mats"]
    metal = m[:, 7] == 1.0
    return {
        "no transcendental lobe (clearcoat and spec_trans 0, or metallic 1)":
            metal | ((m[:, 13] == 0.0) & (m[:, 15] == 0.0)),
        "transmissive (spec_trans = 1)": m[:, 15] == 1.0,
        "metal (metallic = 1)": metal,
        "clearcoat > 0": m[:, 13] > 0.0,
        "inside (eta = 1 / ior)": g["eta"] < 1.0,
    }


def _report(name, exact, close):
    print(f"{name}: {int((~exact).sum())} of {exact.size} cases differ in some bit; "
          f"{int((~close).sum())} beyond 1e-4")


def test_device_bsdf_eval(ctx, golden):
    g = golden("bsdf")
    f, pdf = ctx.bsdf_eval(g["mats"], g["eta"], g["N"], g["V"], g["L"])
    exact = (bits(f) == bits(g["eval_f"])).all(-1) & (bits(pdf) == bits(g["eval_pdf"]))
    close = rel_close(f, g["eval_f"], 1e-4, 1e-7).all(-1) & rel_close(pdf, g["eval_pdf"], 1e-4, 1e-7)
    _report("Eval", exact, close)
    classes = _classes(g)
    for cname, sel in classes.items():
        print(f"  {cname}: {sel.sum()} cases, {exact[sel].mean() * 100:.2f} % bit-exact")
    plain = classes["no transcendental lobe (clearcoat and spec_trans 0, or metallic 1)"]
    assert plain.sum() >= 300
    assert exact[plain].all(), np.nonzero(plain & ~exact)[0][:10]
    assert close.all(), np.nonzero(~close)[0][:10]


def test_device_bsdf_sample(ctx, golden):
    g = golden("bsdf")
    ok, od, col, pdf = ctx.bsdf_sample(g["mats"], g["eta"], g["N"], g["V"], int(g["seed"]), 3)
    assert np.array_equal(ok, g["sample_ok"]), np.nonzero(ok != g["sample_ok"])[0][:10]
    exact = ((bits(od) == bits(g["sample_dir"])).all(-1) & (bits(col) == bits(g["sample_color"])).all(-1)
             & (bits(pdf) == bits(g["sample_pdf"])))
    close = (rel_close(od, g["sample_dir"], 1e-4, 1e-7).all(-1)
             & rel_close(col, g["sample_color"], 1e-4, 1e-7).all(-1)
             & rel_close(pdf, g["sample_pdf"], 1e-4, 1e-7))
    print(f"Sample: returns true on {ok.mean() * 100:.1f} % of cases (equal on all)")
    _report("Sample", exact, close)
    for cname, sel in _classes(g).items():
        print(f"  {cname}: {sel.sum()} cases, {close[sel].mean() * 100:.2f} % within 1e-4")
    assert close.mean() >= 0.995, close.mean()
