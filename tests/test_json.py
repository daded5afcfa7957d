"""On-disk parameter format: the reference's JSON form of arrays
(pyRBMonGPU/json_numpy.py) and of Psi / PsiDeep (Psi.py:8-47, PsiDeep.py:8-46), checked
against files written by the reference's own encoder (tests/golden/psi_json_ref.json).
Bit-exact: JSON carries the doubles' shortest round-trip decimal forms."""
import json
import os

import numpy as np
import pytest

from golden_cases import GOLDEN
from rbmongpu_gb300 import json_numpy as jn

REF = json.load(open(os.path.join(GOLDEN, "psi_json_ref.json")))


def test_encoder_matches_reference_form():
    """Decoding the reference's encoding and encoding it again gives the same JSON."""
    for obj in REF.values():
        assert jn.encode(jn.decode(obj)) == obj


def test_decoder_types():
    d = jn.decode(REF["deep"])
    assert d["b"][0].dtype == np.complex128 and d["connections"][0].dtype == np.uint32
    assert d["alpha"].dtype == np.float64 and d["prefactor"] == 1.0 and d["free_quantum_axis"] is False


gpu = pytest.mark.gpu


@gpu
def test_psi_from_reference_json_and_back():
    import rbmongpu_gb300 as rg
    ref = jn.decode(REF["psi"])
    psi = rg.Psi.from_json(REF["psi"])
    np.testing.assert_array_equal(psi.b, ref["b"])
    np.testing.assert_array_equal(psi.W, ref["W"])
    assert psi.prefactor == ref["prefactor"]
    assert psi.to_json() == REF["psi"]


@gpu
def test_deep_from_reference_json_and_back():
    import rbmongpu_gb300 as rg
    ref = jn.decode(REF["deep"])
    psi = rg.PsiDeep.from_json(REF["deep"])
    for a, b in zip(psi.b, ref["b"]):
        np.testing.assert_array_equal(a, b)
    for a, b in zip(psi.W, ref["W"]):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(psi.final_weights, ref["final_weights"])
    back = jn.decode(psi.to_json())
    for k in ("b", "W", "connections"):
        for a, b in zip(back[k], ref[k]):
            np.testing.assert_array_equal(np.asarray(a), np.asarray(b))
    # a file without final weights loads with ones (PsiDeep.py:42)
    obj = dict(REF["deep"])
    del obj["final_weights"]
    np.testing.assert_array_equal(rg.PsiDeep.from_json(obj).final_weights, np.ones(3))


@gpu
def test_pair_round_trip():
    import rbmongpu_gb300 as rg
    ref = jn.decode(REF["deep"])
    pair = rg.PsiPair(ref["alpha"], ref["beta"], ref["b"], ref["connections"], ref["W"], ref["final_weights"], 1.0)
    again = rg.PsiPair.from_json(pair.to_json())
    np.testing.assert_array_equal(again.params, pair.params)
