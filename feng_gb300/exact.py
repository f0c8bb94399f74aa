"""Closed-form fields used for essential boundary values and error norms.

Each function takes arrays x, y and returns a tuple of component arrays
(scalar fields return a 1-tuple).  They are the manufactured / analytical
solutions of the benchmark problems:

* ``sin_sin``      u = sin(pi x) sin(pi y)  (tests/withLinearSolver/scalarFE.cpp:15-20)
* ``ns_mms``       u = (x^4 y^4, -4/5 x^3 y^5), p = x^2 y^2
                   (tests/withLinearSolver/navier_stokes.cpp:17-31)
* ``kovasznay``    Kovasznay (1948) laminar wake behind a grid, exact steady
                   Navier-Stokes solution for Reynolds number Re.
* ``cavity_lid``   lid-driven cavity: u = (1, 0) on y = y_top, 0 elsewhere.
* ``poiseuille``   plane Poiseuille flow in the channel [0, L] x [0, H]:
                   u = (-dpdx/2 y (H - y), 0), p = -dpdx (L - x)
                   (tests/withLinearSolver/navier_stokes.cpp:177-193,
                   stokes.cpp:166-181).
"""
from __future__ import annotations

import math

import numpy as np


def sin_sin(x, y):
    return (np.sin(np.pi * x) * np.sin(np.pi * y),)


def ns_mms_velocity(x, y):
    return (x**4 * y**4, -4.0 / 5.0 * x**3 * y**5)


def ns_mms_pressure(x, y):
    return (x * x * y * y,)


def kovasznay_lambda(re: float) -> float:
    return re / 2.0 - math.sqrt(re * re / 4.0 + 4.0 * math.pi * math.pi)


def kovasznay_velocity(re: float):
    lam = kovasznay_lambda(re)

    def f(x, y):
        e = np.exp(lam * x)
        return (1.0 - e * np.cos(2 * np.pi * y), lam / (2 * np.pi) * e * np.sin(2 * np.pi * y))

    return f


def kovasznay_pressure(re: float):
    lam = kovasznay_lambda(re)

    def f(x, y):
        return (0.5 * (1.0 - np.exp(2 * lam * x)),)

    return f


def cavity_lid(y_top: float = 1.0, tol: float = 1e-12):
    def f(x, y):
        u = np.where(np.abs(y - y_top) <= tol, 1.0, 0.0)
        return (u, np.zeros_like(u))

    return f


def zero_vector(x, y):
    return (np.zeros_like(x), np.zeros_like(x))


def zero_scalar(x, y):
    return (np.zeros_like(x),)


def poiseuille_velocity(height: float = 1.0, dpdx: float = -1.0):
    def f(x, y):
        return (-dpdx / 2.0 * y * (height - y), np.zeros_like(np.asarray(y, np.float64)))

    return f


def poiseuille_pressure(length: float = 5.0, dpdx: float = -1.0):
    def f(x, y):
        return (-dpdx * (length - x),)

    return f
