"""Closed-form references for the test cases (test infrastructure).

waters_king: start-up Poiseuille flow of an Oldroyd-B fluid (Waters & King's series), which the
reference uses as its own check of the Poiseuille case (data_directory/poiseuille.m:3-57).  The
channel has width h; the body force f drives it from rest; eta is the total viscosity, lam the
relaxation time and beta the viscosity ratio (retardation time beta * lam); density 1."""
import numpy as np


def waters_king(y, t, eta, lam, beta, f, h=1.0, nn=60):
    y1 = np.asarray(y) / h
    t1 = eta * t / (h * h)
    S1 = eta * lam / (h * h)
    S2 = eta * beta * lam / (h * h)
    u = -4.0 * y1 * (y1 - 1.0) + 0j
    for n in range(1, nn + 1):
        N = (2 * n - 1) * np.pi
        aN = 1.0 + S2 * N**2
        bN = np.sqrt(complex(aN**2 - 4.0 * S1 * N**2))
        # exp(-aN t1 / 2S1) (cosh + cN sinh)(bN t1 / 2S1), from exponentials that cannot overflow
        ep = np.exp((-aN + bN) * t1 / (2.0 * S1))
        em = np.exp((-aN - bN) * t1 / (2.0 * S1))
        cN = (1.0 + (S2 - 2.0 * S1) * N**2) / bN
        u = u - 32.0 * np.sin(N * y1) / N**3 * (0.5 * (ep + em) + cN * 0.5 * (ep - em))
    return u.real * f * h * h / (8.0 * eta)
