"""Seeded synthetic initial states (the reference ships no data; its drivers start from noise).

A state holds Gaussian coefficients of amplitude 1e-3*exp(-k/8)*exp(-n/4) for the interior radial point n
and the theta slot k, drawn for psi, T and S in that order from ``numpy.random.default_rng(seed)`` and
laid out like Vecs_to_X (Matrix_Operators.py:529-575); the conductive base state enters the equations
separately (Main.py:201-202)."""
import numpy as np

from .Matrix_Operators import Vecs_to_X


def seeded_state(N_fm, nr, seed, symmetric=False):
    """Flat state of length 3*N_fm*nr; ``seed`` is an int or a numpy Generator (drawn from in place)."""
    rng = seed if isinstance(seed, np.random.Generator) else np.random.default_rng(seed)
    k = np.arange(N_fm)[None, :]
    n = np.arange(nr)[:, None]
    amp = 1e-3 * np.exp(-k / 8.0) * np.exp(-n / 4.0)
    P, T, S = [rng.standard_normal((nr, N_fm)) * amp for _ in range(3)]
    return Vecs_to_X(P, T, S, N_fm, nr, symmetric)
