"""Generate the golden fixtures in this folder from the RBMonGPU reference itself.

Builds seeded inputs with numpy, runs them through ``oracle/_ref/ref_harness`` (the
reference's own host path, compiled from its sources by ``oracle/ref/build_ref.sh``)
and stores inputs and reference outputs together in ``<case>.npz``.

    sh oracle/ref/build_ref.sh && python tests/golden/make_golden.py [case ...]

Needs the reference sources; the committed .npz files are what the tests read.
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
HARNESS = os.path.join(REPO, "oracle", "_ref", "ref_harness")


# ---------------------------------------------------------------- operators
def table(strings, coefs):
    """Padded reference table: types/indices [S, L+1], index -1 terminates a row."""
    L = max(len(s) for s in strings) + 1
    S = len(strings)
    types = np.zeros((S, L), np.int32)
    idx = -np.ones((S, L), np.int32)
    for n, s in enumerate(strings):
        for c, (t, i) in enumerate(s):
            types[n, c] = t
            idx[n, c] = i
    return np.asarray(coefs, np.complex128), types, idx


def tfim_chain(N, J=1.0, h=1.0):
    strings, coefs = [], []
    for i in range(N):
        strings.append([(3, i), (3, (i + 1) % N)])
        coefs.append(-J)
    for i in range(N):
        strings.append([(1, i)])
        coefs.append(-h)
    return table(strings, coefs)


def tfim_square(L, J=1.0, h=1.0):
    strings, coefs = [], []
    for r in range(L):
        for c in range(L):
            i = r * L + c
            strings.append([(3, i), (3, r * L + (c + 1) % L)])
            coefs.append(-J)
            strings.append([(3, i), (3, ((r + 1) % L) * L + c)])
            coefs.append(-J)
    for i in range(L * L):
        strings.append([(1, i)])
        coefs.append(-h)
    return table(strings, coefs)


def mixed_operator(N, rng):
    """Strings with X, Y and Z on random sites, including repeated sites."""
    strings, coefs = [], []
    for _ in range(3 * N):
        k = int(rng.integers(1, 4))
        strings.append([(int(rng.integers(1, 4)), int(rng.integers(0, N))) for _ in range(k)])
        coefs.append(complex(rng.normal(), rng.normal()))
    strings.append([(0, 0)])           # identity column only: a diagonal constant
    coefs.append(0.5)
    return table(strings, coefs)


def identity_op():
    return np.asarray([1.0], np.complex128), np.zeros((1, 1), np.int32), -np.ones((1, 1), np.int32)


# ---------------------------------------------------------------- parameters
def cnormal(rng, shape, sigma):
    return rng.normal(0.0, sigma, shape) + 1j * rng.normal(0.0, sigma, shape)


def deep_connections(N, sizes, conns):
    """Connection pattern (j * delta + i) % n of the reference's new_deep_neural_network."""
    out = []
    for n, m, c in zip([N] + sizes[:-1], sizes, conns):
        delta = 1 if m > n else (n // m if n % m == 0 else c)
        out.append(np.array([[(j * delta + i) % n for j in range(m)] for i in range(c)], np.uint32))
    return out


def write_case(d, meta, arrays):
    with open(os.path.join(d, "meta.txt"), "w") as f:
        for k, v in meta.items():
            f.write(f"{k} {v}\n")
    for k, v in arrays.items():
        np.ascontiguousarray(v).tofile(os.path.join(d, k))


def read_outputs(d):
    out = {}
    with open(os.path.join(d, "out_scalars.txt")) as f:
        for line in f:
            k, v = line.split()
            out["s_" + k] = np.float64(v)
    for name in os.listdir(d):
        if name.startswith("out_") and name.endswith(".bin"):
            key = name[4:-4]
            raw = np.fromfile(os.path.join(d, name), np.uint8)
            if key == "mc_spins":
                out["o_" + key] = raw.view(np.uint64)
            elif key == "mc_logpsi":
                out["o_" + key] = raw.view(np.float64).view(np.complex128)
            else:
                out["o_" + key] = raw.view(np.complex128)
    return out


def op_arrays(prefix, op):
    coef, types, idx = op
    return {prefix + "coef.bin": coef, prefix + "types.bin": types, prefix + "idx.bin": idx}


def run_case(name, meta, arrays, keep):
    with tempfile.TemporaryDirectory() as d:
        write_case(d, meta, arrays)
        subprocess.run([HARNESS, d], check=True)
        out = read_outputs(d)
    payload = {("i_" + k.replace(".bin", "")): v for k, v in arrays.items() if k.replace(".bin", "") in keep}
    payload.update({"m_" + k: np.asarray(v) for k, v in meta.items() if k != "kind"})
    payload["m_kind"] = np.asarray(meta["kind"])
    payload.update(out)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **payload)
    print("wrote", name, sorted(k for k in payload if k.startswith(("s_", "o_"))))


def act_points(rng):
    z = list(cnormal(rng, 24, 1.0)) + list(cnormal(rng, 8, 5.0))
    z += [0.0, 0.0 + 1j, -0.0 - 0.5j, 1e-3 + 1e-3j, -2.0 + 3.0j, 12.0 - 7.0j]
    return np.asarray(z, np.complex128)


def quaxis(meta, arrays, rng, N):
    """free quantum axis: alpha angles of psi and of psi' (alpha' = alpha + N(0, 0.05^2));
    the reference sets beta = alpha (include/quantum_state/PsiBase.hpp:176)."""
    alpha = rng.normal(0, 0.3, N)
    meta["fqa"] = 1
    arrays["alpha.bin"] = alpha
    arrays["pp_alpha.bin"] = alpha + rng.normal(0, 0.05, N)


def rbm_case(name, N, M, sigma, seed, op, hop, unitary, nu, mc=None, normalize=True, ok_count=4, smatrix=False,
             kl=False, ev_extra=False, fqa=False):
    rng = np.random.Generator(np.random.PCG64(seed))
    b = cnormal(rng, M, sigma)
    W = cnormal(rng, (N, M), sigma)
    pb = b + cnormal(rng, M, 1e-3)
    pW = W + cnormal(rng, (N, M), 1e-3)
    ok_spins = rng.integers(0, 2 ** min(N, 62), ok_count, dtype=np.uint64)
    meta = {"kind": "rbm", "N": N, "M": M, "prefactor": 1.0, "normalize": int(normalize),
            "exact": int(N <= 16), "ok": 1, "hsd_unitary": int(unitary), "hsd_nu": nu, "smatrix": int(smatrix),
            "kl": int(kl)}
    if mc:
        meta.update(mc)
    if ev_extra:   # fluctuation_gradient, the operator list [op, hop] and difference
        meta["ev_extra"] = 1
    arrays = {"b.bin": b, "W.bin": W, "pp_b.bin": pb, "pp_W.bin": pW, "ok_spins.bin": ok_spins,
              "act_in.bin": act_points(rng)}
    if fqa:
        quaxis(meta, arrays, rng, N)
    arrays.update(op_arrays("op_", op))
    arrays.update(op_arrays("hop_", hop))
    run_case(name, meta, arrays, keep={k.replace(".bin", "") for k in arrays})


def deep_case(name, kind, N, sizes, conns, sigma, seed, op, hop, unitary, nu, mc=None, dense=False, hsd2=None,
              diag_density=0, ev_extra=False, fqa=False):
    rng = np.random.Generator(np.random.PCG64(seed))
    if dense:
        conn = [np.tile(np.arange(c, dtype=np.uint32)[:, None], (1, m)) for c, m in zip(conns, sizes)]
    else:
        conn = deep_connections(N, sizes, conns)
    meta = {"kind": kind, "N": N, "layers": len(sizes), "prefactor": 1.0, "normalize": 1,
            "exact": 1, "ok": int(kind == "deep"), "hsd_unitary": int(unitary), "hsd_nu": nu}
    arrays = {}
    for l, (m, c) in enumerate(zip(sizes, conns)):
        meta[f"size{l}"] = m
        meta[f"conn{l}"] = c
        w = cnormal(rng, (c, m), sigma)
        bb = cnormal(rng, m, sigma)
        arrays[f"b{l}.bin"] = bb
        arrays[f"W{l}.bin"] = w
        arrays[f"conn{l}.bin"] = conn[l]
        arrays[f"pp_b{l}.bin"] = bb + cnormal(rng, m, 1e-3)
        arrays[f"pp_W{l}.bin"] = w + cnormal(rng, (c, m), 1e-3)
        arrays[f"pp_conn{l}.bin"] = conn[l]
    fw = np.ones(sizes[-1], np.complex128) + cnormal(rng, sizes[-1], sigma)
    arrays["fw.bin"] = fw
    arrays["pp_fw.bin"] = fw + cnormal(rng, sizes[-1], 1e-3)
    arrays["ok_spins.bin"] = rng.integers(0, 2 ** N, 4, dtype=np.uint64)
    if mc:
        meta.update(mc)
    if ev_extra:   # fluctuation_gradient, the operator list [op, hop] and corrected(op, hop)
        meta["ev_extra"] = 1
    if fqa:
        quaxis(meta, arrays, rng, N)
    arrays.update(op_arrays("op_", op))
    arrays.update(op_arrays("hop_", hop))
    if diag_density:
        meta["diag_density"] = diag_density    # DiagDensityOp(sub_system_size) with op_
    if hsd2 is not None:
        # the second-order distance's operator and its square (the reference's expr and
        # expr * expr), the square formed by rbmongpu_gb300.operators.product
        if REPO not in sys.path:
            sys.path.insert(0, REPO)
        from rbmongpu_gb300.operators import product
        meta["hsd2"] = 1
        arrays.update(op_arrays("h2a_", hsd2))
        arrays.update(op_arrays("h2b_", product(hsd2, hsd2)))
    run_case(name, meta, arrays, keep={k.replace(".bin", "") for k in arrays})


def main():
    """Writes every case, or only the cases named on the command line."""
    if not os.path.exists(HARNESS):
        sys.exit("build the reference harness first: sh oracle/ref/build_ref.sh <RBMonGPU checkout>")
    only = set(sys.argv[1:])
    global rbm_case, deep_case
    if only:
        def pick(fn):
            return lambda name, *a, **k: fn(name, *a, **k) if name in only else None
        rbm_case, deep_case = pick(rbm_case), pick(deep_case)
    # N=12, M=24 complex RBM, sigma 0.01, periodic TFIM h=1: exact <H>, gradient, HSD to a
    # copy perturbed by complex N(0, 1e-3^2) under the identity operator (unitary).
    rbm_case("c1_rbm_exact", 12, 24, 0.01, 101, tfim_chain(12, 1.0, 1.0), identity_op(), True, 1.0,
             mc={"mc_samples": 200, "mc_sweeps": 1, "mc_therm": 10, "mc_gradient": 1}, ev_extra=True)
    # small RBM, non-unitary HSD with op = 1j * t * H (the reference's test_distance1 form)
    cf, ty, ix = tfim_chain(6, 1.0, 0.7)
    rbm_case("rbm6_hsd_nonunitary", 6, 12, 0.1, 7, tfim_chain(6, 1.0, 0.7), (1j * 1e-3 * cf, ty, ix), False, 2.0)
    # general Pauli strings (X, Y, Z, repeated sites, identity row)
    rng = np.random.Generator(np.random.PCG64(11))
    mixed = mixed_operator(8, rng)
    rbm_case("rbm8_mixed_operator", 8, 16, 0.2, 12, mixed, mixed, False, 1.0,
             mc={"mc_samples": 100, "mc_sweeps": 2, "mc_therm": 4, "mc_gradient": 1}, ev_extra=True)
    # N=64, M=128 RBM, sigma 0.05, 8x8 periodic TFIM h=3: one reference chain (host path,
    # mt19937(0)) with spins, log psi, accept counts and the MC gradient with the E_k term.
    rbm_case("c2_rbm_mc", 64, 128, 0.05, 102, tfim_square(8, 1.0, 3.0), identity_op(), True, 1.0,
             mc={"mc_samples": 40, "mc_sweeps": 1, "mc_therm": 5, "mc_gradient": 1}, normalize=False)
    # PsiDeep 8 -> [16, 8, 4] with connectivity [4, 2, 4] (the reference's own test net shape)
    deep_case("deep8_sparse", "deep", 8, [16, 8, 4], [4, 2, 4], 0.1, 103, tfim_chain(8), identity_op(), True, 1.0,
              mc={"mc_samples": 60, "mc_sweeps": 1, "mc_therm": 3, "mc_gradient": 1}, ev_extra=True)
    # dense 10 -> 20 -> 10 -> 5 (the layer pattern of the 100->200->100->50 net, scaled down)
    deep_case("deep10_dense", "deep", 10, [20, 10, 5], [10, 20, 10], 0.1, 104, tfim_chain(10), identity_op(),
              True, 1.0, ev_extra=True)
    # get_S_matrix of a small RBM over ExactSummation (the reference's only instantiation)
    # and the KullbackLeibler value and gradient to the perturbed copy (nu = 0.5)
    rbm_case("rbm6_smatrix", 6, 12, 0.3, 13, tfim_chain(6, 1.0, 1.0), identity_op(), True, 0.5, smatrix=True,
             kl=True)
    # second-order distance (PsiDeep with ExactSummation, its only instantiation) for the
    # step generator -i t H, t = 0.02, of the periodic TFIM chain; DiagDensityOp of the
    # first 3 spins with the chain Hamiltonian
    cf, ty, ix = tfim_chain(6, 1.0, 1.0)
    deep_case("deep6_hsd2", "deep", 6, [12, 6], [3, 4], 0.2, 106, tfim_chain(6), identity_op(), True, 1.0,
              hsd2=(-0.02j * cf, ty, ix), diag_density=3)
    # free quantum axis (alpha / beta rotations in the Hilbert-space distance): a small RBM and
    # a small PsiDeep with random alpha, psi' alpha perturbed, the non-unitary step operator
    cf, ty, ix = tfim_chain(6, 1.0, 0.7)
    rbm_case("rbm6_hsd_fqa", 6, 12, 0.1, 17, tfim_chain(6, 1.0, 0.7), (1j * 1e-2 * cf, ty, ix), False, 1.0,
             fqa=True)
    deep_case("deep6_hsd_fqa", "deep", 6, [12, 6], [3, 4], 0.2, 18, tfim_chain(6), (1j * 1e-2 * cf, ty, ix),
              False, 1.0, fqa=True)
    # PsiPair 3 -> [9, 6] connectivity [1, 3] (the reference's test fixture)
    deep_case("pair3", "pair", 3, [9, 6], [1, 3], 0.3, 105, tfim_chain(3), identity_op(), True, 1.0)


if __name__ == "__main__":
    main()
