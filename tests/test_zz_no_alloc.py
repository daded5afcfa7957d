"""The allocation-free exact-summation energy entry point, called through the C ABI.

rbmg_ev_value_exact_noalloc serves callers that cannot call cudaMalloc (frameworks that
own all device memory through their own pool, loops that cannot afford cudaFree's
synchronisation); its scratch is a fixed device array.  Two calls
in a row must agree with rbmg_ev_value on an ExactSummation ensemble (the entry point
that allocates its workspace), within the 1e-5 relative tolerance of the other tests.
This file is collected last so that a first failure here comes after all other tests.
"""
import ctypes as C

import numpy as np
import pytest

import rbmongpu_gb300 as rg
from rbmongpu_gb300 import _lib
from golden_cases import Case

pytestmark = pytest.mark.gpu

RTOL = 1e-5


def test_noalloc_energy_matches_allocating_entry_point_twice():
    c = Case("c1_rbm_exact")
    b, W = c.rbm()
    psi = rg.Psi(np.zeros(c.N), np.zeros(c.N), b, W, c.prefactor, False, True)
    op = rg.Operator(*c.op())
    ref = rg.ExpectationValue()(psi, op, rg.ExactSummation(c.N))
    lib = _lib.lib()
    for _ in range(2):
        out = (C.c_double * 2)()
        rc = lib.rbmg_ev_value_exact_noalloc(psi._h, op._h, c.N, out)
        assert rc == _lib.RBMG_OK, lib.rbmg_last_error().decode()
        got = complex(out[0], out[1])
        assert abs(got - ref) <= RTOL * abs(ref), (got, ref)
    # and against the reference's own value
    assert abs(got - complex(c.s("E_re"), c.s("E_im"))) <= RTOL * abs(ref)


def test_noalloc_energy_with_order_one_weights():
    """Weights of order one, where the FP32 rounding of the device parameters (this entry
    point's log psi comes from them) matters most; still within the 1e-5 tolerance of the
    allocating entry point and of the FP64 restatement."""
    from oracle import pyoracle as po
    rng = np.random.Generator(np.random.PCG64(17))
    N, M = 10, 20
    b = rng.normal(0, 1.0, M) + 1j * rng.normal(0, 1.0, M)
    W = rng.normal(0, 1.0, (N, M)) + 1j * rng.normal(0, 1.0, (N, M))
    psi = rg.Psi(np.zeros(N), np.zeros(N), b, W, 1.0, False, True)
    es = rg.ExactSummation(N)
    psi.normalize(es)
    table = rg.operators.tfim_chain(N, 1.0, 1.0)
    op = rg.Operator(*table)
    ref = rg.ExpectationValue()(psi, op, es)
    _, exact = po.exact_gradient(po.RBM(b, W, psi.prefactor), po.Op(*table))
    lib = _lib.lib()
    for _ in range(2):
        out = (C.c_double * 2)()
        rc = lib.rbmg_ev_value_exact_noalloc(psi._h, op._h, N, out)
        assert rc == _lib.RBMG_OK, lib.rbmg_last_error().decode()
        got = complex(out[0], out[1])
        assert abs(got - ref) <= RTOL * abs(ref), (got, ref)
        assert abs(got - exact) <= RTOL * abs(exact), (got, exact)


def test_noalloc_energy_rejects_sizes_beyond_its_scratch():
    rng = np.random.Generator(np.random.PCG64(3))
    N, M = 15, 16
    psi = rg.Psi(np.zeros(N), np.zeros(N), 0.01 * rng.normal(size=M), 0.01 * rng.normal(size=(N, M)), 1.0)
    op = rg.Operator(*rg.operators.tfim_chain(N))
    out = (C.c_double * 2)()
    rc = _lib.lib().rbmg_ev_value_exact_noalloc(psi._h, op._h, N, out)
    assert rc == _lib.RBMG_EINVAL
    assert b"14" in _lib.lib().rbmg_last_error()
