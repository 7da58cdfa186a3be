"""Shared helpers for the parity tests."""
import numpy as np

from rendertoy_gb300.scenes import Scene


def scene_from_fixture(g) -> Scene:
    return Scene(verts=g["verts"], norms=g["norms"], tri_mesh=g["tri_mesh"], mesh_mat=g["mesh_mat"],
                 mesh_smooth=g["mesh_smooth"], mats=g["mats"], sky=g["sky"], ground=g["ground"],
                 camera=g["camera"], name="fixture")


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def same_bits(a, b):
    """Bit-equal arrays, except that NaN payloads need not agree (NaN
    positions must)."""
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    na, nb = np.isnan(a), np.isnan(b)
    return bool(np.array_equal(na, nb) and np.array_equal(bits(a)[~na], bits(b)[~nb]))


def rel_close(a, b, rtol, atol=0.0):
    """Elementwise |a - b| <= rtol * max(|a|, |b|) + atol, NaN == NaN."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    both_nan = np.isnan(a) & np.isnan(b)
    with np.errstate(invalid="ignore"):
        ok = np.abs(a - b) <= rtol * np.maximum(np.abs(a), np.abs(b)) + atol
    return ok | both_nan | (a == b)


def relmse(x, ref, eps=1e-2):
    x = np.asarray(x, np.float64)
    ref = np.asarray(ref, np.float64)
    m = np.isfinite(x) & np.isfinite(ref)
    return float(np.mean(((x - ref) ** 2 / (ref ** 2 + eps))[m]))
