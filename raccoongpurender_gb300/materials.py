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
