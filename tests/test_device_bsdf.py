"""The device principled BSDF on its own (rtx_bsdf_eval / rtx_bsdf_sample,
the code the shading kernel inlines) against the 3,000 golden
PrincipledBSDF::Eval / Sample cases the reference's own sources produced
(src/material.cpp:143-204, 206-295; tests/golden/bsdf.npz): random materials
with metallic 0 / 1 / random, spec_trans 0 / 1 / random (so refraction and
total internal reflection occur), clearcoat on and off, rays from inside and
outside.

Both sides use the same arithmetic in the same order with --fmad=false, so
results agree bit for bit except where a transcendental (sqrtf is exact;
powf, expf, cosf, sinf, logf are not) rounds one ulp apart between the CUDA
math library and the host C library.  The count of cases that differ in any
bit is printed; every case must still agree within 1e-4 relative, and each
material class must be >= 99 % bit-exact.
"""
import numpy as np
import pytest

from helpers import bits, rel_close

pytestmark = pytest.mark.gpu


def _classes(g):
    m = g["mats"]
    return {
        "all": np.ones(len(m), bool),
        "transmissive (spec_trans = 1)": m[:, 15] == 1.0,
        "metal (metallic = 1)": m[:, 7] == 1.0,
        "clearcoat > 0": m[:, 13] > 0.0,
        "inside (eta = 1 / ior)": g["eta"] < 1.0,
    }


def _report(name, exact, close, classes):
    print(f"{name}: {int((~exact).sum())} of {exact.size} cases differ in some bit; "
          f"{int((~close).sum())} beyond 1e-4")
    for cname, sel in classes.items():
        if sel.any():
            frac = exact[sel].mean()
            print(f"  {cname}: {sel.sum()} cases, {frac * 100:.2f} % bit-exact")
            assert frac >= 0.99, (name, cname, frac)
    assert close.all(), (name, np.nonzero(~close)[0][:10])


def test_device_bsdf_eval(ctx, golden):
    g = golden("bsdf")
    f, pdf = ctx.bsdf_eval(g["mats"], g["eta"], g["N"], g["V"], g["L"])
    exact = (bits(f) == bits(g["eval_f"])).all(-1) & (bits(pdf) == bits(g["eval_pdf"]))
    close = rel_close(f, g["eval_f"], 1e-4, 1e-7).all(-1) & rel_close(pdf, g["eval_pdf"], 1e-4, 1e-7)
    _report("Eval", exact, close, _classes(g))


def test_device_bsdf_sample(ctx, golden):
    g = golden("bsdf")
    ok, od, col, pdf = ctx.bsdf_sample(g["mats"], g["eta"], g["N"], g["V"], int(g["seed"]), 3)
    assert np.array_equal(ok, g["sample_ok"]), np.nonzero(ok != g["sample_ok"])[0][:10]
    exact = ((bits(od) == bits(g["sample_dir"])).all(-1) & (bits(col) == bits(g["sample_color"])).all(-1)
             & (bits(pdf) == bits(g["sample_pdf"])))
    close = (rel_close(od, g["sample_dir"], 1e-4, 1e-7).all(-1)
             & rel_close(col, g["sample_color"], 1e-4, 1e-7).all(-1)
             & rel_close(pdf, g["sample_pdf"], 1e-4, 1e-7))
    print(f"Sample: ok fraction {ok.mean():.3f}")
    _report("Sample", exact, close, _classes(g))
