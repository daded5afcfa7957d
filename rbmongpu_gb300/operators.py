"""Operator tables for common lattice Hamiltonians, in the reference's padded layout
(coefficients [S], pauli_types [S, L], pauli_indices [S, L]; types 0=I 1=X 2=Y 3=Z,
index -1 ends a string; include/operator/Operator.hpp:30-88).

The reference builds these from QuantumExpression objects
(source/operator/Operator.cpp:12-61); these builders produce the same tables directly.
"""
import numpy as np

I, X, Y, Z = 0, 1, 2, 3


def table(strings, coefficients):
    """strings: list of [(pauli_type, site), ...]; returns (coef, types, indices)."""
    L = max((len(s) for s in strings), default=0) + 1
    S = len(strings)
    types = np.zeros((S, L), np.int32)
    idx = -np.ones((S, L), np.int32)
    for n, s in enumerate(strings):
        for c, (t, i) in enumerate(s):
            types[n, c] = t
            idx[n, c] = i
    return np.asarray(coefficients, np.complex128), types, idx


def tfim_chain(N, J=1.0, h=1.0):
    """Periodic 1D transverse-field Ising chain H = -J sum z_i z_{i+1} - h sum x_i."""
    strings = [[(Z, i), (Z, (i + 1) % N)] for i in range(N)] + [[(X, i)] for i in range(N)]
    return table(strings, [-J] * N + [-h] * N)


def tfim_square(L, J=1.0, h=1.0):
    """Periodic L x L transverse-field Ising model (2 L^2 bonds + L^2 fields)."""
    strings, coefs = [], []
    for r in range(L):
        for c in range(L):
            i = r * L + c
            strings.append([(Z, i), (Z, r * L + (c + 1) % L)])
            strings.append([(Z, i), (Z, ((r + 1) % L) * L + c)])
            coefs += [-J, -J]
    strings += [[(X, i)] for i in range(L * L)]
    coefs += [-h] * (L * L)
    return table(strings, coefs)


def heisenberg_chain(N, J=1.0):
    """Periodic Heisenberg chain J sum (x x + y y + z z)."""
    strings, coefs = [], []
    for i in range(N):
        k = (i + 1) % N
        for t in (X, Y, Z):
            strings.append([(t, i), (t, k)])
            coefs.append(J)
    return table(strings, coefs)


def identity():
    """The identity operator (one string with no Pauli factor)."""
    return np.asarray([1.0], np.complex128), np.zeros((1, 1), np.int32), -np.ones((1, 1), np.int32)


def scaled(op, factor):
    coef, types, idx = op
    return np.asarray(coef) * factor, types, idx


# single-site Pauli products: _MUL[a][b] = (phase, c) with sigma_a sigma_b = phase sigma_c
_MUL = [[(1, I), (1, X), (1, Y), (1, Z)],
        [(1, X), (1, I), (1j, Z), (-1j, Y)],
        [(1, Y), (-1j, Z), (1, I), (1j, X)],
        [(1, Z), (1j, Y), (-1j, X), (1, I)]]


def _strings(op):
    """(coefficient, {site: pauli}) per row, repeated sites multiplied in row order."""
    coef, types, idx = op
    out = []
    for n in range(len(coef)):
        c, sites = complex(coef[n]), {}
        for t, i in zip(types[n], idx[n]):
            if i < 0:
                break
            if t == I:
                continue
            ph, r = _MUL[sites.get(int(i), I)][int(t)]
            c *= ph
            if r == I:
                sites.pop(int(i), None)
            else:
                sites[int(i)] = r
        out.append((c, sites))
    return out


def _merge(terms):
    acc = {}
    for c, sites in terms:
        key = tuple(sorted(sites.items()))
        acc[key] = acc.get(key, 0) + c
    keys = [k for k, v in acc.items() if v != 0]
    if not keys:
        return identity()[0] * 0, identity()[1], identity()[2]
    return table([[(t, i) for i, t in k] for k in keys], [acc[k] for k in keys])


def product(op_a, op_b):
    """The operator product A B of two operator tables (the reference multiplies
    QuantumExpression objects, e.g. expr * expr for the second-order distance), equal
    strings merged, sites in ascending order."""
    terms = []
    for ca, sa in _strings(op_a):
        for cb, sb in _strings(op_b):
            c, sites = ca * cb, dict(sa)
            for i, t in sb.items():
                ph, r = _MUL[sites.get(i, I)][t]
                c *= ph
                if r == I:
                    sites.pop(i, None)
                else:
                    sites[i] = r
            terms.append((c, sites))
    return _merge(terms)
