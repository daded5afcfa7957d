"""ctypes view of the CPU restatement in oracle/liboracle.so.

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` and by
the benchmark's CPU-baseline leg, as the checker.  The product package never
imports it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

OR_RNG_MT19937, OR_RNG_PHILOX = 0, 1
OR_PREC_REF64, OR_PREC_GPU32 = 0, 1
OR_PSI_RBM, OR_PSI_DEEP, OR_PSI_PAIR = 0, 1, 2

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_up = C.POINTER(C.c_uint)
_u64p = C.POINTER(C.c_uint64)


class _Op(C.Structure):
    _fields_ = [("S", C.c_int), ("L", C.c_int), ("coef", _dp), ("types", _ip), ("idx", _ip)]


class _Psi(C.Structure):
    _fields_ = [
        ("kind", C.c_int), ("N", C.c_int), ("prefactor", C.c_double),
        ("M", C.c_int), ("b", _dp), ("W", _dp),
        ("num_layers", C.c_int), ("size", C.c_int * 3), ("conn", C.c_int * 3),
        ("lhs_conn", _up * 3), ("lhs_w", _dp * 3), ("bias", _dp * 3), ("final_w", _dp),
        ("lhs_w_im", _dp * 3), ("bias_im", _dp * 3), ("final_w_im", _dp),
        ("translational_invariance", C.c_int),
        ("free_quantum_axis", C.c_int), ("alpha", _dp), ("beta", _dp),
    ]


class _McCfg(C.Structure):
    _fields_ = [
        ("total_chains", C.c_int), ("chain_begin", C.c_int), ("num_chains", C.c_int),
        ("samples_per_chain", C.c_int), ("num_sweeps", C.c_int), ("num_therm", C.c_int),
        ("rng", C.c_int), ("seed", C.c_uint64), ("prec", C.c_int),
        ("fast_sweep_tries", C.c_int), ("total_z", C.c_int), ("sector", C.c_int),
        ("state_spins", _u64p), ("state_rng", _u64p), ("resume", C.c_int),
    ]


def build():
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, "oracle.c")):
            build()
        L = C.CDLL(LIB_PATH)
        L.or_philox_word.restype = C.c_uint32
        L.or_philox_word.argtypes = [C.c_uint64, C.c_uint32, C.c_uint64]
        L.or_lc_re_f32.restype = C.c_float
        L.or_lc_re_f32.argtypes = [C.c_float, C.c_float]
        L.or_expf_det.restype = C.c_float
        L.or_expf_det.argtypes = [C.c_float]
        L.or_logf_det.restype = C.c_float
        L.or_logf_det.argtypes = [C.c_float]
        L.or_exact_norm.restype = C.c_double
        L.or_exact_hsd.restype = C.c_double
        L.or_samples_hsd.restype = C.c_double
        L.or_num_params.restype = C.c_int
        _lib = L
    return _lib


def _c128(a):
    return np.ascontiguousarray(np.asarray(a, np.complex128))


def _ptr(a, t=_dp):
    return a.ctypes.data_as(t)


class Op:
    """Reference operator table (coefficients [S], pauli types / indices [S, L])."""

    def __init__(self, coef, types, idx):
        self.coef = _c128(coef)
        self.types = np.ascontiguousarray(types, np.int32)
        self.idx = np.ascontiguousarray(idx, np.int32)
        self.c = _Op(len(self.coef), self.types.shape[1], _ptr(self.coef.view(np.float64)),
                     _ptr(self.types, _ip), _ptr(self.idx, _ip))


class RBM:
    def __init__(self, b, W, prefactor=1.0, alpha=None, beta=None, free_quantum_axis=False):
        self.b = _c128(b)
        self.W = _c128(W)
        self.N, self.M = self.W.shape
        self.c = _Psi()
        self.c.kind = OR_PSI_RBM
        self.c.N = self.N
        self.c.M = self.M
        self.c.prefactor = prefactor
        self.c.b = _ptr(self.b.view(np.float64))
        self.c.W = _ptr(self.W.view(np.float64))
        _set_quaxis(self, alpha, beta, free_quantum_axis)

    @property
    def num_params(self):
        return 2 * self.N + self.M + self.N * self.M


def _set_quaxis(obj, alpha, beta, free_quantum_axis):
    """alpha / beta rotation angles [N] (real) and the free-quantum-axis flag of a psi."""
    obj.alpha = np.ascontiguousarray(np.zeros(obj.N) if alpha is None else np.real(alpha), np.float64)
    obj.beta = np.ascontiguousarray(obj.alpha if beta is None else np.real(beta), np.float64)
    obj.c.alpha = _ptr(obj.alpha)
    obj.c.beta = _ptr(obj.beta)
    obj.c.free_quantum_axis = int(bool(free_quantum_axis))
    return obj


class Deep:
    """PsiDeep (pair=False) or PsiPair (pair=True) from complex per-layer arrays."""

    def __init__(self, N, biases, connections, weights, final_weights, prefactor=1.0, pair=False,
                 translational_invariance=False, alpha=None, beta=None, free_quantum_axis=False):
        self.N = N
        self.keep = []
        self.c = _Psi()
        self.c.kind = OR_PSI_PAIR if pair else OR_PSI_DEEP
        self.c.N = N
        self.c.prefactor = prefactor
        self.c.num_layers = len(biases)
        self.c.translational_invariance = int(translational_invariance)
        _set_quaxis(self, alpha, beta, free_quantum_axis)

        def hold(a):
            self.keep.append(a)
            return a

        for l, (b, cn, w) in enumerate(zip(biases, connections, weights)):
            cn = hold(np.ascontiguousarray(cn, np.uint32))
            self.c.size[l] = len(b)
            self.c.conn[l] = cn.shape[0]
            self.c.lhs_conn[l] = _ptr(cn, _up)
            if pair:
                self.c.lhs_w[l] = _ptr(hold(np.ascontiguousarray(np.real(w), np.float64)))
                self.c.bias[l] = _ptr(hold(np.ascontiguousarray(np.real(b), np.float64)))
                self.c.lhs_w_im[l] = _ptr(hold(np.ascontiguousarray(np.imag(w), np.float64)))
                self.c.bias_im[l] = _ptr(hold(np.ascontiguousarray(np.imag(b), np.float64)))
            else:
                self.c.lhs_w[l] = _ptr(hold(_c128(w)).view(np.float64))
                self.c.bias[l] = _ptr(hold(_c128(b)).view(np.float64))
        if pair:
            self.c.final_w = _ptr(hold(np.ascontiguousarray(np.real(final_weights), np.float64)))
            self.c.final_w_im = _ptr(hold(np.ascontiguousarray(np.imag(final_weights), np.float64)))
        else:
            self.c.final_w = _ptr(hold(_c128(final_weights)).view(np.float64))

    @property
    def num_params(self):
        return lib().or_num_params(C.byref(self.c))


def nwords(N):
    return (N + 63) // 64


def spins_array(configs, N):
    """uint64 bitsets [count, nwords] from python ints or a uint64 array."""
    nw = nwords(N)
    out = np.zeros((len(configs), nw), np.uint64)
    for t, c in enumerate(configs):
        c = int(c)
        for k in range(nw):
            out[t, k] = (c >> (64 * k)) & 0xFFFFFFFFFFFFFFFF
    return out


def log_psi(psi, spins):
    out = np.zeros(2)
    s = np.ascontiguousarray(spins, np.uint64)
    lib().or_log_psi(C.byref(psi.c), _ptr(s, _u64p), _ptr(out))
    return complex(out[0], out[1])


def O_k(psi, spins):
    P = psi.num_params
    out = np.zeros(2 * P)
    s = np.ascontiguousarray(spins, np.uint64)
    lib().or_O_k(C.byref(psi.c), _ptr(s, _u64p), _ptr(out))
    return out.view(np.complex128)


def s_matrix(psi, spins, weights=None, centered=False):
    """get_S_matrix (source/network_functions/S_matrix.cu:10-53): S[k, k'] = sum_s c_s
    O_k(s) conj(O_k'(s)) / sum_s c_s over the configurations `spins` [n][nwords], with
    c_s = 1 as the reference has it (its ExactSummation weight is not applied) or the
    given weights; centered subtracts <O> <O>^dagger (the covariance of SR)."""
    O = np.array([O_k(psi, s) for s in np.asarray(spins, np.uint64)])
    c = np.ones(len(O)) if weights is None else np.asarray(weights, np.float64)
    c = c / c.sum()
    if centered:   # rows centred first: the covariance is not the difference of two large sums
        O = O - c @ O
    return np.einsum("s,sk,sl->kl", c, O, O.conj())


def hsd_2nd_order(psi, psi_prime, op, op2, spins, weights=None):
    """distance_2nd_order (source/network_functions/HilbertSpaceDistance_2nd_order.cu:14-95)
    over the configurations `spins` with weights (exact summation: prefactor^2 |psi|^2;
    None: 1 per sample, Monte Carlo)."""
    om = np.zeros(len(spins), complex)
    nn = np.zeros(len(spins))
    pr = np.zeros(len(spins))
    for n, s in enumerate(np.asarray(spins, np.uint64)):
        lp, lpp = log_psi(psi, s), log_psi(psi_prime, s)
        e1, e2 = local_energy(psi, op, s, lp), local_energy(psi, op2, s, lp)
        x = e1 + 0.5 * (e2 - e1 * e1)
        om[n] = np.exp(x + np.conj(lpp - lp))
        nn[n] = np.exp(2.0 * x.real)
        pr[n] = np.exp(2.0 * (lpp - lp).real)
    w = np.ones(len(spins)) if weights is None else np.asarray(weights, np.float64)
    o, a, b = (w * om).sum(), (w * nn).sum(), (w * pr).sum()
    return np.sqrt(1.0 - abs(o) ** 2 / (a * b))


def kl(psi, psi_prime, spins, weights=None, nu=1.0, gradient=True):
    """KullbackLeibler value / gradient (source/network_functions/KullbackLeibler.cu:14-137):
    D = log psi' - log psi, value = sqrt(<|D|^2> - |<D>|^2), grad_k = (<D O_k'*> -
    <D><O_k'*>) / max(value, 1e-6)^nu; weights None: 1 per sample (Monte Carlo), else the
    exact-summation weights prefactor^2 |psi|^2."""
    sp = np.asarray(spins, np.uint64)
    D = np.array([log_psi(psi_prime, s) - log_psi(psi, s) for s in sp])
    w = np.ones(len(sp)) / len(sp) if weights is None else np.asarray(weights, np.float64)
    m = (w * D).sum()
    value = np.sqrt((w * np.abs(D) ** 2).sum() - abs(m) ** 2)
    if not gradient:
        return None, value
    O = np.array([O_k(psi_prime, s) for s in sp])
    g = ((w * D) @ O.conj() - m * (w @ O.conj())) / max(value, 1e-6) ** nu
    return g, value


def diag_density(psi, op, spins, na, weights=None):
    """DiagDensityOp (source/network_functions/DiagDensityOp.cu:12-50): sum of
    weight |E_loc|^2 per configuration of the first na spins; weights None: 1 per sample
    and the sums divided by the sample count (Monte Carlo), else the exact-summation
    weights prefactor^2 |psi|^2."""
    out = np.zeros(1 << na)
    sp = np.asarray(spins, np.uint64)
    for n, s in enumerate(sp):
        e = local_energy(psi, op, s)
        w = 1.0 if weights is None else weights[n]
        out[int(s[0]) & ((1 << na) - 1)] += w * abs(e) ** 2
    return out / len(sp) if weights is None else out


def local_energy(psi, op, spins, lp=None):
    s = np.ascontiguousarray(spins, np.uint64)
    if lp is None:
        lp = log_psi(psi, s)
    lpa = np.array([lp.real, lp.imag])
    out = np.zeros(2)
    lib().or_local_energy(C.byref(psi.c), C.byref(op.c), _ptr(s, _u64p), _ptr(lpa), _ptr(out))
    return complex(out[0], out[1])


def E_k(psi, op, spins, lp=None):
    """E_k(s) = sum_n e_n(s) O_k(s'_n), the local energy's parameter vector
    (Operator.hpp:145-179 foreach_E_k_s_prime) of one configuration."""
    s = np.ascontiguousarray(spins, np.uint64)
    if lp is None:
        lp = log_psi(psi, s)
    lpa = np.array([lp.real, lp.imag])
    acc = np.zeros(2 * psi.num_params)
    lib().or_E_k_accumulate(C.byref(psi.c), C.byref(op.c), _ptr(s, _u64p), _ptr(lpa), C.c_double(1.0), _ptr(acc))
    return acc.view(np.complex128)


def exact_configs(psi):
    """Every configuration of N <= 16 spins with the reference's ExactSummation weight
    prefactor^2 |psi(s)|^2 (include/quantum_state/Psi.hpp:134-137); averages are sums of weight x value (its
    get_num_steps is 1)."""
    s = np.arange(2 ** psi.N, dtype=np.uint64)[:, None]
    lp = np.array([log_psi(psi, x) for x in s])
    return s, np.exp(2.0 * (np.log(psi.c.prefactor) + lp.real))


def _avg_weights(n, weights):
    """per-sample factors of the averages: weight / num_steps (MonteCarloLoop: 1 / n)"""
    return np.full(n, 1.0 / n) if weights is None else np.asarray(weights, np.float64)


def fluctuation_gradient(psi, op, spins, weights=None):
    """ExpectationValue::fluctuation_gradient (ExpectationValue.cu:258-348): the gradient of
    sigma = sqrt(<|E|^2> - |<E>|^2),
      1 / (2 sigma) (2 conj(<E* E_k> - <E>* <E_k>) - 2 <E>* <E O_k*> + 2 <O_k>* (2 |<E>|^2 - <|E|^2>))."""
    sp = np.asarray(spins, np.uint64)
    c = _avg_weights(len(sp), weights)
    lp = [log_psi(psi, x) for x in sp]
    E = np.array([local_energy(psi, op, x, l) for x, l in zip(sp, lp)])
    O = np.array([O_k(psi, x) for x in sp])
    Ek = np.array([E_k(psi, op, x, l) for x, l in zip(sp, lp)])
    Ea = c @ E
    E2 = c @ np.abs(E) ** 2
    sigma = np.sqrt(E2 - abs(Ea) ** 2)
    EEk = c @ (np.conj(E)[:, None] * Ek)
    Oa = c @ O
    EO = c @ (E[:, None] * np.conj(O))
    Eka = c @ Ek
    return (2 * np.conj(EEk - np.conj(Ea) * Eka) - 2 * np.conj(Ea) * EO
            + 2 * np.conj(Oa) * (2 * abs(Ea) ** 2 - E2)) / (2 * sigma)


def ev_list(psi, ops, spins, weights=None):
    """ExpectationValue::operator() of an operator list (ExpectationValue.cu:448-518): every
    operator's <E_loc> over the same configurations."""
    sp = np.asarray(spins, np.uint64)
    c = _avg_weights(len(sp), weights)
    lp = [log_psi(psi, x) for x in sp]
    return np.array([c @ np.array([local_energy(psi, o, x, l) for x, l in zip(sp, lp)]) for o in ops])


def ev_difference(psi, psi_prime, ops, spins, weights=None):
    """ExpectationValue::difference (ExpectationValue.cu:350-446): for each operator
    <E'> - <r E> / <r>, E' the local energy under psi_prime, r = |psi / psi_prime|^2."""
    sp = np.asarray(spins, np.uint64)
    c = _avg_weights(len(sp), weights)
    lp = [log_psi(psi, x) for x in sp]
    lpp = [log_psi(psi_prime, x) for x in sp]
    r = np.exp(2.0 * (np.real(lp) - np.real(lpp)))
    out = []
    for o in ops:
        a = c @ np.array([local_energy(psi_prime, o, x, l) for x, l in zip(sp, lpp)])
        b = c @ (r * np.array([local_energy(psi, o, x, l) for x, l in zip(sp, lp)]))
        out.append(a - b / (c @ r))
    return np.array(out)


def ev_corrected(psi, op, spins, weights=None):
    """ExpectationValue::corrected (ExpectationValue.cu:76-127).  The reference evaluates its
    first operator twice (operator2 is not used): with E the local energy, it returns
    (<E> / <a>, <a>), a = exp(2 Im E + Re(E E - E))."""
    sp = np.asarray(spins, np.uint64)
    c = _avg_weights(len(sp), weights)
    E = np.array([local_energy(psi, op, x) for x in sp])
    a = np.exp(2.0 * E.imag + (E * E - E).real)
    return (c @ E) / (c @ a), c @ a


def exact_norm(psi):
    return lib().or_exact_norm(C.byref(psi.c))


def psi_vector(psi):
    out = np.zeros(2 << psi.N)
    lib().or_psi_vector(C.byref(psi.c), _ptr(out))
    return out.view(np.complex128)


def exact_fluctuation(psi, op):
    E = np.zeros(2)
    sig = C.c_double()
    lib().or_exact_fluctuation(C.byref(psi.c), C.byref(op.c), _ptr(E), C.byref(sig))
    return sig.value, complex(E[0], E[1])


def exact_gradient(psi, op):
    P = psi.num_params
    g = np.zeros(2 * P)
    E = np.zeros(2)
    lib().or_exact_gradient(C.byref(psi.c), C.byref(op.c), _ptr(g), _ptr(E))
    return g.view(np.complex128), complex(E[0], E[1])


def exact_hsd(psi, psi_prime, op, is_unitary, nu=1.0, gradient=True):
    P = psi_prime.num_params
    g = np.zeros(2 * P) if gradient else None
    d = lib().or_exact_hsd(C.byref(psi.c), C.byref(psi_prime.c), C.byref(op.c), int(is_unitary),
                           C.c_double(nu), _ptr(g) if gradient else None)
    return (g.view(np.complex128) if gradient else None), d


def samples_gradient(psi, op, spins):
    s = np.ascontiguousarray(spins, np.uint64)
    P = psi.num_params
    g = np.zeros(2 * P)
    E = np.zeros(2)
    lib().or_samples_gradient(C.byref(psi.c), C.byref(op.c), len(s), _ptr(s, _u64p), _ptr(g), _ptr(E))
    return g.view(np.complex128), complex(E[0], E[1])


def samples_hsd(psi, psi_prime, op, is_unitary, spins, nu=1.0, gradient=True):
    s = np.ascontiguousarray(spins, np.uint64)
    P = psi_prime.num_params
    g = np.zeros(2 * P) if gradient else None
    d = lib().or_samples_hsd(C.byref(psi.c), C.byref(psi_prime.c), C.byref(op.c), int(is_unitary), len(s),
                             _ptr(s, _u64p), C.c_double(nu), _ptr(g) if gradient else None)
    return (g.view(np.complex128) if gradient else None), d


def mc_run(psi, op, num_chains, samples_per_chain, num_sweeps, num_therm, rng=OR_RNG_PHILOX, seed=0,
           prec=OR_PREC_GPU32, chain_begin=0, total_chains=None, total_z=False, sector=0, fast_sweep_tries=0,
           want_eloc=True, state=None):
    """Runs chains and returns (spins [samples, chains, nwords], log_psi, eloc, accepts, rejects).
    state: optional (spins [chains, nwords] uint64, rng [chains] uint64, resume flag list) carried
    between calls."""
    nw = nwords(psi.N)
    cfg = _McCfg(total_chains or num_chains, chain_begin, num_chains, samples_per_chain, num_sweeps, num_therm,
                 rng, seed, prec, fast_sweep_tries, int(total_z), sector)
    if state is not None:
        cfg.state_spins = _ptr(state[0], _u64p)
        cfg.state_rng = _ptr(state[1], _u64p)
        cfg.resume = int(state[2][0])
        state[2][0] = 1
    spins = np.zeros((samples_per_chain, num_chains, nw), np.uint64)
    lp = np.zeros((samples_per_chain, num_chains, 2))
    el = np.zeros((samples_per_chain, num_chains, 2))
    acc = np.zeros(num_chains, np.uint64)
    rej = np.zeros(num_chains, np.uint64)
    r = lib().or_mc_run(C.byref(psi.c), C.byref(op.c) if op is not None else None, C.byref(cfg),
                        _ptr(spins, _u64p), _ptr(lp), _ptr(el) if (want_eloc and op is not None) else None,
                        _ptr(acc, _u64p), _ptr(rej, _u64p))
    if r != 0:
        raise ValueError("oracle mc_run: unsupported configuration")
    return (spins, lp.view(np.complex128)[..., 0], el.view(np.complex128)[..., 0], acc, rej)


def logcosh(z):
    out = np.zeros(2)
    lib().or_logcosh(C.c_double(z.real), C.c_double(z.imag), _ptr(out))
    return complex(out[0], out[1])


def tanh(z):
    out = np.zeros(2)
    lib().or_tanh(C.c_double(z.real), C.c_double(z.imag), _ptr(out))
    return complex(out[0], out[1])


def philox_word(seed, walker, index):
    return lib().or_philox_word(seed, walker, index)


def mt_words(seed, count):
    out = np.zeros(count, np.uint32)
    lib().or_mt_words(C.c_uint32(seed), count, _ptr(out, C.POINTER(C.c_uint32)))
    return out


def expf_det(x):
    return lib().or_expf_det(C.c_float(x))


def lc_re_f32(x, y):
    return lib().or_lc_re_f32(C.c_float(x), C.c_float(y))


def div_pos_f32(num, den):
    """The FMA-only quotient of the Metropolis test (device_math.cuh::div_pos), elementwise."""
    num = np.ascontiguousarray(num, np.float32)
    den = np.ascontiguousarray(den, np.float32)
    out = np.empty_like(num)
    fp = C.POINTER(C.c_float)
    lib().or_div_pos_f32_n(num.ctypes.data_as(fp), den.ctypes.data_as(fp), out.ctypes.data_as(fp),
                           C.c_long(num.size))
    return out


def logf_det(x):
    """The deterministic FP32 log of the proposal's softmax (device_math.cuh::logf_det)."""
    return lib().or_logf_det(C.c_float(x))


def learned_replay(W, trace, seed, walker_base=0):
    """FP32 replay of the frozen learned Metropolis-Hastings steps recorded by
    Chain.learned_trace (rbmongpu_gb300/csrc/proposal.cu learned_draw_kernel and
    learned_accept_kernel), fed the device's initial angles and its logits: returns the
    replay's moves (site, len, logq), acceptances, spins after every step and the final
    Philox positions."""
    W = np.asarray(W, np.complex128)
    N, M = W.shape
    Wr = np.ascontiguousarray(W.real.astype(np.float32))
    Wi = np.ascontiguousarray(W.imag.astype(np.float32))
    steps, B = trace["site"].shape
    Mpad = trace["re0"].shape[1]
    nw = nwords(N)
    out = dict(site=np.zeros((steps, B), np.int32), len=np.zeros((steps, B), np.int32),
               logq=np.zeros((steps, B), np.float32), spins=np.zeros((steps, B, nw), np.uint64),
               accepted=np.zeros((steps, B), np.uint8), rng_end=np.zeros(B, np.uint64))
    fp = C.POINTER(C.c_float)
    ip = C.POINTER(C.c_int)
    arr = lambda a, t: np.ascontiguousarray(a).ctypes.data_as(t)   # noqa: E731
    keep = {k: np.ascontiguousarray(trace[k]) for k in ("spins0", "rng0", "theta0", "re0", "logits0", "logits_prop")}
    r = lib().or_learned_replay(
        N, M, Mpad, arr(Wr, fp), arr(Wi, fp), B, steps, C.c_uint64(seed), C.c_uint32(walker_base),
        arr(keep["spins0"], _u64p), arr(keep["rng0"], _u64p), arr(keep["theta0"], fp), arr(keep["re0"], fp),
        arr(keep["logits0"], fp), arr(keep["logits_prop"], fp), arr(out["site"], ip), arr(out["len"], ip),
        arr(out["logq"], fp), arr(out["spins"], _u64p), out["accepted"].ctypes.data_as(C.POINTER(C.c_uint8)),
        arr(out["rng_end"], _u64p))
    if r != 0:
        raise ValueError(f"or_learned_replay failed ({r})")
    return out


def _replay_walker(args):
    b, W, prefactor, w, samples, therm, seed, total = args
    spins, _, _, acc, rej = mc_run(RBM(b, W, prefactor), None, 1, samples, 1, therm, seed=seed, chain_begin=w,
                                   total_chains=total, want_eloc=False)
    return spins[:, 0], int(acc[0]), int(rej[0])


def mc_run_walkers(b, W, prefactor, walkers, samples, therm, seed, total_chains, workers=None):
    """FP32 replays (Philox stream, the CUDA sampler's operation order) of the given walkers
    of a `total_chains`-walker MonteCarloLoop pass, one sweep per sample, in a process pool
    (spawn context, so it is safe after CUDA was initialised in the caller).  Returns
    (spins [samples, len(walkers), nwords], accepts [len(walkers)], rejects)."""
    import multiprocessing as mp
    import os
    jobs = [(np.asarray(b), np.asarray(W), prefactor, int(w), samples, therm, seed, total_chains) for w in walkers]
    with mp.get_context("spawn").Pool(workers or min(len(jobs), os.cpu_count() or 1)) as pool:
        out = pool.map(_replay_walker, jobs)
    spins = np.stack([o[0] for o in out], axis=1)
    return spins, np.array([o[1] for o in out], np.uint64), np.array([o[2] for o in out], np.uint64)
