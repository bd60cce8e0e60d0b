"""The reference's analytic solution of a thick-walled Mooney-Rivlin cylinder
under inflation and extension (test infrastructure: the known answer that pins
the assembly and Newton path; nothing in the library imports it).

Restates FiniteElasticity_CylinderAnalyticCalculate and
FINITE_ELASTICITY_CYLINDER_ANALYTIC_FUNC_EVALUATE
(finite_elasticity_routines.f90:491-602) with the reference's parameter
names: inner pressure PIN, outer pressure POUT, axial stretch LAMBDA, twist
TSI, outer radius A1, inner radius A2, Mooney-Rivlin C1, C2.  The deformation
is r = MU(R) R with MU^2 = (1 + K / R^2) / LAMBDA, K = A1^2 (LAMBDA MU1^2 - 1),
theta' = theta + TSI LAMBDA Z, z = LAMBDA Z, where MU1 (the outer radial
stretch) is the root of the reference's residual function, found by its
Newton iteration with a forward-difference derivative (step 1e-5), step
halving and relative tolerance 1e-12 (:515-546).

The reference's boundary conditions for this solution
(FiniteElasticity_BoundaryConditionsAnalyticCalculate, :132-484) apply PIN on
the inner surface and POUT on the outer surface as incremented surface
pressures, fix z on the bottom (z = 0) and on the top (z = LAMBDA H), and fix
x (y) on the bottom nodes with x = 0 (y = 0); they impose no twist, so the
solution is compared with TSI = 0.

Pressure: the reference's P (:578-579) is the multiplier of the split
sigma = 2 C1 B + 2 C2 (I1 B - B^2) + P I.  The library's pressure dof p is
the hydrostatic part of sigma = dev(sigma_bar) + p I (the stress of
finite_elasticity_routines.f90:4413-4414 / 4441-4442), so
p = P + tr(sigma_bar) / 3 = P + (2/3)(C1 I1 + 2 C2 I2), with I1, I2 the
invariants of B at that point; `library_pressure` returns that value.
"""
from __future__ import annotations

import math

import numpy as np


def residual_function(mu1, pin, pout, lam, tsi, a1, a2, c1, c2):
    """FINITE_ELASTICITY_CYLINDER_ANALYTIC_FUNC_EVALUATE
    (finite_elasticity_routines.f90:581-602), term for term."""
    k = a1 ** 2 * (lam * mu1 ** 2 - 1.0)
    mu = math.sqrt(1.0 / lam * (1.0 + k / a2 ** 2))
    return (2.0 * (c1 / lam ** 2 / mu ** 2 + c2 * (1.0 / lam ** 2 + 1.0 / mu ** 2 + tsi ** 2 * a2 ** 2))
            + pout - (c1 / lam + c2 * lam) * (1.0 / lam / mu1 ** 2 - a2 ** 2 / (a2 ** 2 + k) + 2 * math.log(mu / mu1))
            + c1 * tsi ** 2 * lam * (a2 ** 2 - a1 ** 2)
            - 2.0 * (c1 / lam ** 2 / mu ** 2 + c2 * (1.0 / lam ** 2 + 1.0 / mu ** 2 + tsi ** 2 * a2 ** 2)) + pin)


def solve_mu1(pin, pout, lam, tsi, a1, a2, c1, c2, step=1e-5, reltol=1e-12):
    """Newton iteration of FiniteElasticity_CylinderAnalyticCalculate
    (:515-546): initial guess 1, forward-difference derivative, the step
    halved until |F| decreases (failure below a step of 1e-3), stop when
    the relative step DELTA / (1 + MU1) is below RELTOL.  The reference
    compares the signed DELTA in both tests, so a negative Newton step ends
    its loop after one step, before the root is reached; this restatement
    compares |DELTA|, so that it returns the root the routine is meant to
    find (the function value there is checked by the tests)."""
    args = (pin, pout, lam, tsi, a1, a2, c1, c2)
    zero_tol = 5.0 * np.finfo(float).eps
    mu1 = 1.0
    for _ in range(200):
        f = residual_function(mu1, *args)
        df = (residual_function(mu1 + step, *args) - f) / step
        delta = -f / df
        f2 = residual_function(mu1 + delta, *args)
        while True:
            if abs(f2) < abs(f) or abs(f2) < zero_tol:
                mu1 += delta
                break
            if abs(delta) < 1e-3:
                raise RuntimeError("cylinder analytic solution: Newton for MU1 failed to converge")
            delta /= 2.0
            f2 = residual_function(mu1 + delta, *args)
        if abs(delta) / (1.0 + mu1) < reltol:
            return mu1
    raise RuntimeError("cylinder analytic solution: no convergence in 200 iterations")


class CylinderSolution:
    """Deformed position and pressure of every material point of the tube."""

    def __init__(self, pin, pout, lam, a1, a2, c1, c2, tsi=0.0):
        self.pin, self.pout, self.lam, self.tsi = pin, pout, lam, tsi
        self.a1, self.a2, self.c1, self.c2 = a1, a2, c1, c2
        self.mu1 = solve_mu1(pin, pout, lam, tsi, a1, a2, c1, c2)
        self.k = a1 ** 2 * (lam * self.mu1 ** 2 - 1.0)

    def mu(self, R):
        return np.sqrt(1.0 / self.lam * (1.0 + self.k / R ** 2))

    def deformed(self, X):
        """Deformed coordinates (3, n) of undeformed points X (3, n)
        (finite_elasticity_routines.f90:566-576)."""
        R = np.hypot(X[0], X[1])
        th = np.arctan2(X[1], X[0])
        r = self.mu(R) * R
        tht = th + self.tsi * self.lam * X[2]
        return np.stack([r * np.cos(tht), r * np.sin(tht), self.lam * X[2]])

    def reference_pressure(self, R):
        """The reference's P (finite_elasticity_routines.f90:578-579)."""
        c1, c2, lam, tsi, mu1, k = self.c1, self.c2, self.lam, self.tsi, self.mu1, self.k
        mu = self.mu(R)
        return (self.pout - (c1 / lam + c2 * lam) * (1.0 / lam / mu1 ** 2 - R ** 2 / (R ** 2 + k)
                                                     + np.log(mu ** 2 / mu1 ** 2))
                + c1 * tsi ** 2 * lam * (R ** 2 - self.a1 ** 2)
                - 2.0 * (c1 / lam ** 2 / mu ** 2 + c2 * (1.0 / lam ** 2 + 1.0 / mu ** 2 + tsi ** 2 * R ** 2)))

    def library_pressure(self, R):
        """The library's pressure dof at radius R (TSI = 0): P + (2/3)(C1 I1 +
        2 C2 I2) with principal stretches (1 / (LAMBDA MU), MU, LAMBDA)."""
        if self.tsi != 0.0:
            raise ValueError("library_pressure is stated for TSI = 0")
        mu = self.mu(R)
        s2 = np.stack([1.0 / (self.lam * mu) ** 2, mu ** 2, np.full_like(mu, self.lam ** 2)])
        i1 = s2.sum(axis=0)
        i2 = s2[0] * s2[1] + s2[1] * s2[2] + s2[0] * s2[2]
        return self.reference_pressure(R) + (2.0 / 3.0) * (self.c1 * i1 + 2.0 * self.c2 * i2)
