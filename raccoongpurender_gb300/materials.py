"""Material records of the reference (common/material_type.hpp:28-63), as
dicts accepted by :class:`raccoongpurender_gb300.SceneManager`.  Defaults are
the reference defaults."""
from __future__ import annotations

LAMBERTIAN = 1
SPECULAR = 2
DIELECTRIC = 3
WARD = 4
HOMOGENEOUS_VOLUME = 5


def lambertian(le=(0.0, 0.0, 0.0), r=(1.0, 1.0, 1.0), back_emission: bool = False) -> dict:
    return dict(type=LAMBERTIAN, le=tuple(map(float, le)), r=tuple(map(float, r)), back_emission=int(back_emission))


def specular() -> dict:
    return dict(type=SPECULAR)


def dielectric() -> dict:
    return dict(type=DIELECTRIC)


def ward(alpha: float = 0.1, reflectance=(1.0, 1.0, 1.0), edgetint=(1.0, 1.0, 1.0), falloff: float = 0.5) -> dict:
    return dict(type=WARD, alpha=float(alpha), r=tuple(map(float, reflectance)),
                edgetint=tuple(map(float, edgetint)), falloff=float(falloff))


def homogeneous_volume(c: float = 1.0, r=(1.0, 1.0, 1.0)) -> dict:
    return dict(type=HOMOGENEOUS_VOLUME, c=float(c), r=tuple(map(float, r)))


# numpy layout of struct rgr_material (include/rgr.h), for large per-primitive arrays
import numpy as _np  # noqa: E402

MATERIAL_DTYPE = _np.dtype([("type", "<i4"), ("back_emission", "<i4"), ("le", "<f4", 3), ("r", "<f4", 3),
                            ("edgetint", "<f4", 3), ("alpha", "<f4"), ("falloff", "<f4"), ("c", "<f4")])
assert MATERIAL_DTYPE.itemsize == 56  # sizeof(rgr_material)


def as_array(mats) -> _np.ndarray:
    """Per-primitive materials as a MATERIAL_DTYPE array (from a list of the
    dicts above, or an array already in that layout)."""
    if isinstance(mats, _np.ndarray) and mats.dtype == MATERIAL_DTYPE:
        return _np.ascontiguousarray(mats)
    out = _np.zeros(len(mats), MATERIAL_DTYPE)
    for i, m in enumerate(mats):
        out[i]["type"] = m["type"]
        out[i]["back_emission"] = int(m.get("back_emission", 0))
        out[i]["le"] = m.get("le", (0.0, 0.0, 0.0))
        out[i]["r"] = m.get("r", (1.0, 1.0, 1.0))
        out[i]["edgetint"] = m.get("edgetint", (1.0, 1.0, 1.0))
        out[i]["alpha"] = m.get("alpha", 0.1)
        out[i]["falloff"] = m.get("falloff", 0.5)
        out[i]["c"] = m.get("c", 1.0)
    return out


def random_mix(n: int, rng) -> _np.ndarray:
    """Per-primitive material mix of the full-render configuration: 50 %
    Lambertian (albedo U[0.1, 0.9]^3), 35 % Ward (alpha U[0.05, 0.5], specular
    0.04), 15 % dielectric, drawn from `rng`."""
    u = rng.random(n)
    alb = 0.1 + 0.8 * rng.random((n, 3))
    alpha = 0.05 + 0.45 * rng.random(n)
    out = _np.zeros(n, MATERIAL_DTYPE)
    lam = u < 0.5
    wrd = (u >= 0.5) & (u < 0.85)
    out["type"] = _np.where(lam, LAMBERTIAN, _np.where(wrd, WARD, DIELECTRIC))
    out["r"] = _np.where(lam[:, None], alb, 0.04)
    out["edgetint"] = _np.where(wrd[:, None], 0.04, 1.0)
    out["alpha"] = _np.where(wrd, alpha, 0.1)
    out["falloff"] = 0.5
    out["c"] = 1.0
    return out
