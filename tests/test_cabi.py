"""The C-ABI library loads without a GPU and exports every symbol that
include/rbmg.h declares; host-side logic that needs no device."""
import os
import re

import numpy as np

from rbmongpu_gb300 import _lib, operators

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "rbmg.h")


def declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"RBMG_API\s+(?:const\s+char\*|int)\s+(rbmg_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = _lib.lib()
    names = declared()
    assert len(names) >= 40
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(_lib.SIGNATURES), "python binding and header disagree"


def test_version_and_error_strings_without_gpu():
    lib = _lib.lib()
    assert lib.rbmg_version().decode().startswith("rbmg")
    assert isinstance(lib.rbmg_last_error(), bytes)


def test_argument_validation_fails_loudly_without_touching_the_device():
    import ctypes as C
    lib = _lib.lib()
    h = C.c_void_p()
    # num_samples not a multiple of the chain count: rejected before any CUDA call
    assert lib.rbmg_mc_create(10, 1, 0, 3, 0, C.byref(h)) == _lib.RBMG_EINVAL
    assert b"multiple" in lib.rbmg_last_error()
    assert lib.rbmg_exact_create(0, C.byref(h)) == _lib.RBMG_EINVAL
    # a fixed sample set whose configuration sets a bit at or beyond N
    bad = (C.c_uint64 * 2)(1, 1 << 10)
    assert lib.rbmg_samples_create(10, 2, bad, C.byref(h)) == _lib.RBMG_EINVAL
    assert b"beyond N" in lib.rbmg_last_error()
    out = (C.c_double * 2)()
    assert lib.rbmg_activation(0.3, -0.2, out) == _lib.RBMG_OK


def test_activation_is_the_reference_rational_function():
    from oracle import pyoracle as po
    import rbmongpu_gb300 as rg
    for z in [0.1 + 0.2j, -1.5 + 0.3j, 0.0, 4.0 - 2.0j]:
        assert abs(rg.activation_function(z) - po.logcosh(z)) < 1e-14


def test_operator_tables():
    coef, types, idx = operators.tfim_chain(5, 1.0, 0.5)
    assert types.shape == (10, 3) and idx.shape == (10, 3)
    assert (idx[:, -1] == -1).all()
    assert np.allclose(coef[:5], -1.0) and np.allclose(coef[5:], -0.5)
    c2, t2, i2 = operators.tfim_square(4)
    assert len(c2) == 3 * 16


def test_spins_lattice_shifts():
    """Spins.shift_2d (include/Spins.h:287-332) on an L x L row-major lattice is the cyclic
    roll by (shift_i, shift_j); shift_vertical alone rolls whole rows."""
    from rbmongpu_gb300 import Spins
    rng = np.random.default_rng(2)
    for L in (3, 4, 5, 8):
        N = L * L
        for _ in range(30):
            c = int(rng.integers(0, 2 ** min(N, 62)))
            si, sj = int(rng.integers(0, L)), int(rng.integers(0, L))
            bits = np.array([(c >> i) & 1 for i in range(N)]).reshape(L, L)

            def word(a):
                return sum(int(b) << i for i, b in enumerate(a.reshape(-1)))

            assert Spins(c, N).shift_2d(si, sj, L, L).configuration == word(np.roll(bits, (si, sj), axis=(0, 1)))
            assert Spins(c, N).shift_vertical(si, L, L).configuration == word(np.roll(bits, si, axis=0))
