"""Hidden angles from scratch on the tensor cores (rbmg_psi_angles, angles_tc.cu) against
the FP64 sum b + s W, for every way the hidden units split into 256-wide chunks and spin
counts up to 256.

Tolerance: 1e-5 of the largest angle (the complex64 path's tolerance; the BF16 hi / mid /
lo parts carry W to 24 bits and the sums run in FP32)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N,M,count", [(12, 24, 70), (100, 400, 300), (200, 576, 129), (256, 64, 128),
                                       (33, 300, 1)])
def test_angles_match_fp64_sum(N, M, count):
    import rbmongpu_gb300 as rg
    rng = np.random.default_rng(N + M)
    b = 0.1 * (rng.normal(size=M) + 1j * rng.normal(size=M))
    W = 0.1 * (rng.normal(size=(N, M)) + 1j * rng.normal(size=(N, M)))
    psi = rg.Psi(np.zeros(N), np.zeros(N), b, W, 1.0, False, True)
    nw = (N + 63) // 64
    words = rng.integers(0, 2 ** 63, (count, nw), dtype=np.uint64) | rng.integers(0, 2, (count, nw), dtype=np.uint64)
    if N % 64:
        words[:, -1] &= np.uint64((1 << (N % 64)) - 1)
    th = psi.angles(words)
    bits = (words[:, np.arange(N) // 64] >> (np.arange(N) % 64).astype(np.uint64)) & np.uint64(1)
    s = np.where(bits == 1, 1.0, -1.0)
    # the psi computes with complex64 parameters, as the GPU stores them
    b32 = b.astype(np.complex64).astype(np.complex128)
    W32 = W.astype(np.complex64).astype(np.complex128)
    ref = b32 + s @ W32
    assert th.shape == (count, M)
    err = np.abs(th - ref).max() / np.abs(ref).max()
    assert err < 1e-5, err


def test_angles_follow_parameter_updates():
    """The tensor-core operands are rebuilt when the parameters change (set_params and the
    device optimiser)."""
    import rbmongpu_gb300 as rg
    rng = np.random.default_rng(3)
    N, M = 20, 40
    b = 0.1 * (rng.normal(size=M) + 1j * rng.normal(size=M))
    W = 0.1 * (rng.normal(size=(N, M)) + 1j * rng.normal(size=(N, M)))
    psi = rg.Psi(np.zeros(N), np.zeros(N), b, W, 1.0, False, True)
    words = rng.integers(0, 2 ** N, (16, 1), dtype=np.uint64)
    psi.W = 2.0 * W
    bits = (words[:, [0] * N] >> np.arange(N).astype(np.uint64)) & np.uint64(1)
    s = np.where(bits == 1, 1.0, -1.0)
    ref = b.astype(np.complex64) + s @ (2.0 * W).astype(np.complex64).astype(np.complex128)
    assert np.abs(psi.angles(words) - ref).max() / np.abs(ref).max() < 1e-5
