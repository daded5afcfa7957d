"""Python classes with the names, arguments and results of RBMonGPU's pybind11 module
(pyRBMonGPU/main.cpp:45-614) and its Python veneer (pyRBMonGPU/Psi.py, PsiDeep.py,
PsiPair.py), implemented over the C ABI of include/rbmg.h.

Every computation runs in the CUDA library; the ``gpu`` arguments are accepted for
signature compatibility only.
"""
import ctypes as C
import json
import math

import numpy as np

from ._lib import RbmgError, call, lib

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_u64p = C.POINTER(C.c_uint64)


def _c128(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.complex128))


def _f64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def _p(a, t=_dp):
    return a.ctypes.data_as(t)


def _handle():
    return C.c_void_p()


def nwords(N):
    return (N + 63) // 64


def spins_to_words(spins, N):
    """Accepts a Spins, a python int bit pattern, or a uint64 word array."""
    if isinstance(spins, Spins):
        return spins.words()
    if isinstance(spins, (int, np.integer)):
        v = int(spins)
        return np.array([(v >> (64 * k)) & 0xFFFFFFFFFFFFFFFF for k in range(nwords(N))], np.uint64)
    w = np.ascontiguousarray(np.asarray(spins, dtype=np.uint64)).reshape(-1)
    if w.size != nwords(N):
        raise ValueError("spin configuration has the wrong number of words")
    return w


# --------------------------------------------------------------------- helpers
def setDevice(device):
    call("rbmg_set_device", int(device))


def start_profiling():
    call("rbmg_profiler_start")


def stop_profiling():
    call("rbmg_profiler_stop")


def activation_function(z):
    """The reference's rational log-cosh (include/quantum_state/psi_functions.hpp:49-57)."""
    z = complex(z)
    out = np.zeros(2)
    call("rbmg_activation", z.real, z.imag, _p(out))
    return complex(out[0], out[1])


class Spins:
    """Bit-packed spin configuration: bit i set <=> s_i = +1 (include/Spins.h:222-333)."""

    def __init__(self, configuration, num_spins):
        self.N = int(num_spins)
        mask = (1 << self.N) - 1
        self.configuration = int(configuration) & mask

    def array(self, num_spins=None):
        n = self.N if num_spins is None else num_spins
        return np.array([1.0 if (self.configuration >> i) & 1 else -1.0 for i in range(n)])

    def flip(self, position):
        return Spins(self.configuration ^ (1 << position), self.N)

    def rotate_left(self, shift, N):
        c = self.configuration
        return Spins(((c << shift) | (c >> (N - shift))) & ((1 << N) - 1), N)

    def hamming_distance(self, other):
        return bin(self.configuration ^ other.configuration).count("1")

    # lattice shifts of an nrows x ncols configuration, row-major (include/Spins.h:287-332).
    # The reference forms its column masks in 32-bit arithmetic, which is exact up to 32
    # spins; here the masks are exact for every size.
    def shift_vertical(self, shift, nrows, ncols):
        c, n = self.configuration, nrows * ncols
        return Spins((c << (shift * ncols)) | (c >> ((nrows - shift) * ncols)), n)

    def _columns(self, first, count, nrows, ncols):
        row = ((1 << count) - 1) << first
        mask = 0
        for i in range(nrows):
            mask |= row << (i * ncols)
        return Spins(self.configuration & mask, nrows * ncols)

    def shift_horizontal(self, shift, nrows, ncols):
        # select_left_columns(nrows - shift) | select_right_columns(shift) moved up a row
        # (Spins.h:314-325; the reference counts the left columns with nrows)
        tmp = self.rotate_left(shift, nrows * ncols)
        left = tmp._columns(ncols - (nrows - shift), nrows - shift, nrows, ncols)
        right = tmp._columns(0, shift, nrows, ncols).shift_vertical(nrows - 1, nrows, ncols)
        return Spins(left.configuration | right.configuration, nrows * ncols)

    def shift_2d(self, shift_i, shift_j, nrows, ncols):
        """Spins.h:327-332: the configuration moved by shift_i rows and shift_j columns."""
        return self.shift_vertical(shift_i, nrows, ncols).shift_horizontal(shift_j, nrows, ncols)

    def words(self):
        return spins_to_words(self.configuration, self.N)


# --------------------------------------------------------------------- states
class _PsiBase:
    _h = None

    def __del__(self):
        h, self._h = self._h, None
        if h is not None and lib is not None:
            try:
                lib().rbmg_psi_destroy(h)
            except Exception:
                pass

    @property
    def N(self):
        n = C.c_int()
        call("rbmg_psi_shape", self._h, C.byref(n), None, None)
        return n.value

    @property
    def num_params(self):
        p = C.c_int()
        call("rbmg_psi_shape", self._h, None, None, C.byref(p))
        return p.value

    @property
    def params(self):
        out = np.zeros(self.num_params, np.complex128)
        call("rbmg_psi_get_params", self._h, _p(out.view(np.float64)))
        return out

    @params.setter
    def params(self, new_params):
        v = _c128(new_params)
        if v.size != self.num_params:
            raise ValueError("params has the wrong length")
        call("rbmg_psi_set_params", self._h, _p(v.view(np.float64)))

    @property
    def prefactor(self):
        v = C.c_double()
        call("rbmg_psi_get_prefactor", self._h, C.byref(v))
        return v.value

    @prefactor.setter
    def prefactor(self, value):
        call("rbmg_psi_set_prefactor", self._h, float(value))

    @property
    def alpha(self):
        return self.params[: self.N].real.copy()

    @property
    def beta(self):
        return self.params[self.N: 2 * self.N].real.copy()

    @property
    def gpu(self):
        return True

    @property
    def free_quantum_axis(self):
        v = C.c_int()
        call("rbmg_psi_free_quantum_axis", self._h, C.byref(v))
        return bool(v.value)

    def _vector(self):
        out = np.zeros(1 << self.N, np.complex128)
        call("rbmg_psi_vector", self._h, _p(out.view(np.float64)))
        return out

    @property
    def vector(self):
        # the alpha / beta rotations of pyRBMonGPU/Psi.py:62-74 are built with QuantumExpression
        # (not bundled); the vector is the plain amplitude list, exact where alpha = beta = 0
        return self._vector()

    def norm(self, exact_summation):
        v = C.c_double()
        call("rbmg_psi_norm", self._h, exact_summation._h, C.byref(v))
        return v.value

    def normalize(self, exact_summation):
        """pyRBMonGPU/Psi.py:54-55 (PsiDeep.py:55-57 resets the prefactor to 1 first)."""
        if isinstance(self, PsiDeep):
            self.prefactor = 1.0
        self.prefactor = self.prefactor / self.norm(exact_summation)

    def copy(self):
        h = _handle()
        call("rbmg_psi_copy", self._h, C.byref(h))
        obj = object.__new__(type(self))
        obj.__dict__.update(self.__dict__)
        obj._h = h
        return obj

    def __pos__(self):
        return self.copy()

    def log_psi_s(self, spins):
        w = spins_to_words(spins, self.N)
        out = np.zeros(2)
        call("rbmg_psi_log_psi", self._h, 1, _p(w, _u64p), _p(out))
        return complex(out[0], out[1])

    def angles(self, spins_words):
        """Extension (complex RBM): hidden angles theta = b + s W of configurations (uint64
        words [count][nwords]) -> complex [count][M], built on the tensor cores."""
        w = np.ascontiguousarray(spins_words, np.uint64).reshape(-1, nwords(self.N))
        out = np.zeros(2 * len(w) * self.M)
        call("rbmg_psi_angles", self._h, len(w), _p(w, _u64p), _p(out))
        return out.view(np.complex128).reshape(len(w), self.M)

    def log_psi_batch(self, spins_words):
        w = np.ascontiguousarray(spins_words, np.uint64).reshape(-1, nwords(self.N))
        out = np.zeros(2 * len(w))
        call("rbmg_psi_log_psi", self._h, len(w), _p(w, _u64p), _p(out))
        return out.view(np.complex128)


class Psi(_PsiBase):
    """Complex RBM: Psi(alpha, beta, b, W, prefactor, free_quantum_axis, gpu)
    (include/quantum_state/Psi.hpp:220-238)."""

    def __init__(self, alpha, beta, b, W, prefactor=1.0, free_quantum_axis=False, gpu=True):
        b = _c128(b)
        W = _c128(W)
        N, M = W.shape
        if b.shape != (M,):
            raise ValueError("b must have M entries")
        alpha = _f64(alpha) if alpha is not None else np.zeros(N)
        beta = _f64(beta) if beta is not None else np.zeros(N)
        h = _handle()
        call("rbmg_psi_create", N, M, _p(alpha), _p(beta), _p(b.view(np.float64)), _p(W.view(np.float64)),
             float(prefactor), int(bool(free_quantum_axis)), C.byref(h))
        self._h = h

    @property
    def M(self):
        m = C.c_int()
        call("rbmg_psi_shape", self._h, None, C.byref(m), None)
        return m.value

    @property
    def num_angles(self):
        return self.M

    @property
    def b(self):
        N, M = self.N, self.M
        return self.params[2 * N: 2 * N + M].copy()

    @b.setter
    def b(self, value):
        p = self.params
        N, M = self.N, self.M
        p[2 * N: 2 * N + M] = _c128(value)
        self.params = p

    @property
    def W(self):
        N, M = self.N, self.M
        return self.params[2 * N + M:].reshape(N, M).copy()

    @W.setter
    def W(self, value):
        p = self.params
        N, M = self.N, self.M
        p[2 * N + M:] = _c128(value).reshape(-1)
        self.params = p

    def to_json(self):
        """pyRBMonGPU/Psi.py:8-22: the parameters in the reference's JSON form."""
        from .json_numpy import encode
        return encode(dict(type="Psi", alpha=self.alpha, beta=self.beta, b=self.b, W=self.W,
                           prefactor=self.prefactor))

    @staticmethod
    def from_json(obj, gpu=True):
        """pyRBMonGPU/Psi.py:38-47 (arrays in the reference's JSON form or as numpy arrays)."""
        from .json_numpy import decode
        o = decode(obj)
        return Psi(np.asarray(o["alpha"]).real, np.asarray(o["beta"]).real, o["b"], o["W"], o["prefactor"], False,
                   gpu)


class PsiDeep(_PsiBase):
    """Sparse feed-forward net (include/quantum_state/PsiDeep.hpp:339-400):
    PsiDeep(alpha, beta, b_list, connections_list, W_list, final_weights, prefactor,
    free_quantum_axis, gpu).  PsiPair subclasses it with two real nets."""

    _pair = 0
    # lattice extents for a translation-invariant net (PsiDeep.hpp:80-81, main.cpp:112-113);
    # the reference stores them and its only use of them is commented out, so they are kept
    # here as plain attributes
    N_i = 0
    N_j = 0

    def __init__(self, alpha, beta, b, connections, W, final_weights, prefactor=1.0, free_quantum_axis=False,
                 gpu=True):
        bl = [_c128(x) for x in b]
        cl = [np.ascontiguousarray(np.asarray(c), dtype=np.uint32) for c in connections]
        wl = [_c128(w) for w in W]
        fw = _c128(final_weights)
        L = len(bl)
        N = len(np.asarray(alpha)) if alpha is not None else int(max(int(cl[0].max()) + 1, 1))
        sizes = (C.c_int * L)(*[len(x) for x in bl])
        conns = (C.c_int * L)(*[c.shape[0] for c in cl])
        for l in range(L):
            if cl[l].shape != (conns[l], sizes[l]) or wl[l].shape != (conns[l], sizes[l]):
                raise ValueError(f"layer {l}: connections and weights must be [connectivity, size]")
        cptr = (C.POINTER(C.c_uint32) * L)(*[c.ctypes.data_as(C.POINTER(C.c_uint32)) for c in cl])
        bptr = (_dp * L)(*[_p(x.view(np.float64)) for x in bl])
        wptr = (_dp * L)(*[_p(x.view(np.float64)) for x in wl])
        alpha = _f64(alpha) if alpha is not None else np.zeros(N)
        beta = _f64(beta) if beta is not None else np.zeros(N)
        h = _handle()
        call("rbmg_psi_deep_create", N, L, sizes, conns, cptr, bptr, wptr, _p(fw.view(np.float64)), _p(alpha),
             _p(beta), float(prefactor), int(bool(free_quantum_axis)), self._pair, C.byref(h))
        self._h = h
        self._shapes = [(int(conns[l]), int(sizes[l])) for l in range(L)]
        self._connections = [c.copy() for c in cl]
        self._ti = False

    @property
    def translational_invariance(self):
        return self._ti

    @translational_invariance.setter
    def translational_invariance(self, on):
        call("rbmg_psi_set_translational_invariance", self._h, int(bool(on)))
        self._ti = bool(on)

    def _split(self):
        p = self.params[2 * self.N:]
        out, k = [], 0
        for conn, size in self._shapes:
            b = p[k: k + size]
            k += size
            w = p[k: k + conn * size].reshape(conn, size)
            k += conn * size
            out.append((b, w))
        return out, p[k:]

    @property
    def b(self):
        return [b.copy() for b, _ in self._split()[0]]

    @property
    def W(self):
        return [w.copy() for _, w in self._split()[0]]

    @property
    def connections(self):
        return [c.copy() for c in self._connections]

    @property
    def final_weights(self):
        return self._split()[1].copy()

    @property
    def first_layer_params_slice(self):
        conn, size = self._shapes[0]
        return slice(2 * self.N, 2 * self.N + conn * size + size)


def _deep_to_json(self, kind):
    """pyRBMonGPU/PsiDeep.py:8-24 (PsiPair.py alike)."""
    from .json_numpy import encode
    return encode(dict(type=kind, alpha=self.alpha, beta=self.beta, b=list(self.b), connections=list(self.connections),
                       W=list(self.W), final_weights=self.final_weights, prefactor=self.prefactor,
                       free_quantum_axis=self.free_quantum_axis))


def _deep_from_json(cls, obj, gpu):
    """pyRBMonGPU/PsiDeep.py:27-46: final_weights default to ones of the last layer's size."""
    from .json_numpy import decode
    o = decode(obj)
    fw = o["final_weights"] if "final_weights" in o else np.ones(np.asarray(o["W"][-1]).shape[-1])
    return cls(np.asarray(o["alpha"]).real, np.asarray(o["beta"]).real, o["b"], o["connections"], o["W"], fw,
               o["prefactor"], bool(o.get("free_quantum_axis", False)), gpu)


PsiDeep.to_json = lambda self: _deep_to_json(self, "PsiDeep")
PsiDeep.from_json = staticmethod(lambda obj, gpu=True: _deep_from_json(PsiDeep, obj, gpu))


class PsiPair(PsiDeep):
    """Two real PsiDeep nets for Re / Im log psi (include/quantum_state/PsiPair.hpp:166-205)."""

    _pair = 1


PsiPair.to_json = lambda self: _deep_to_json(self, "PsiPair")
PsiPair.from_json = staticmethod(lambda obj, gpu=True: _deep_from_json(PsiPair, obj, gpu))


# --------------------------------------------------------------------- operator
class Operator:
    """Pauli-string sum as the reference's padded table (include/operator/Operator.hpp:212-227).

    Operator(coefficients[S], pauli_types[S, L], pauli_indices[S, L], gpu); types 0=I 1=X 2=Y 3=Z,
    index -1 ends a string.  An object with a ``to_table()`` method returning the same three
    arrays is accepted in place of the tables (the reference's PauliExpression overload).
    """

    def __init__(self, coefficients, pauli_types=None, pauli_indices=None, gpu=True):
        if pauli_types is None or isinstance(pauli_types, bool):
            coefficients, pauli_types, pauli_indices = coefficients.to_table()
        coef = _c128(coefficients).reshape(-1)
        types = np.ascontiguousarray(np.asarray(pauli_types), dtype=np.int32)
        idx = np.ascontiguousarray(np.asarray(pauli_indices), dtype=np.int32)
        if types.ndim != 2 or types.shape != idx.shape or types.shape[0] != coef.size:
            raise ValueError("pauli_types / pauli_indices must be [num_strings, max_string_length]")
        h = _handle()
        call("rbmg_operator_create", types.shape[0], types.shape[1], _p(coef.view(np.float64)), _p(types, _ip),
             _p(idx, _ip), C.byref(h))
        self._h = h

    def __del__(self):
        h, self._h = getattr(self, "_h", None), None
        if h is not None:
            try:
                lib().rbmg_operator_destroy(h)
            except Exception:
                pass

    def _shape(self):
        s, l = C.c_int(), C.c_int()
        call("rbmg_operator_shape", self._h, C.byref(s), C.byref(l))
        return s.value, l.value

    @property
    def num_strings(self):
        return self._shape()[0]

    @property
    def max_string_length(self):
        return self._shape()[1]

    def _tables(self):
        S, L = self._shape()
        c = np.zeros(S, np.complex128)
        t = np.zeros((S, L), np.int32)
        i = np.zeros((S, L), np.int32)
        call("rbmg_operator_tables", self._h, _p(c.view(np.float64)), _p(t, _ip), _p(i, _ip))
        return c, t, i

    @property
    def coefficients(self):
        return self._tables()[0]

    @property
    def pauli_types(self):
        return self._tables()[1]

    @property
    def pauli_indices(self):
        return self._tables()[2]

    @property
    def gpu(self):
        return True


# --------------------------------------------------------------------- ensembles
class _Ensemble:
    _h = None

    def __del__(self):
        h, self._h = self._h, None
        if h is not None:
            try:
                lib().rbmg_ensemble_destroy(h)
            except Exception:
                pass

    @property
    def num_steps(self):
        n = C.c_uint64()
        call("rbmg_ensemble_num_steps", self._h, C.byref(n))
        return n.value

    def samples(self, psi, operator=None, log_psi=True):
        """(spins words [num_steps, nwords], log psi [num_steps] or None, E_loc or None) of one
        foreach pass."""
        n = self.num_steps
        nw = nwords(psi.N)
        sp = np.zeros((n, nw), np.uint64)
        lp = np.zeros(2 * n) if log_psi else None
        el = np.zeros(2 * n) if operator is not None else None
        call("rbmg_ensemble_samples", self._h, psi._h, operator._h if operator is not None else None,
             _p(sp, _u64p), _p(lp) if lp is not None else None, _p(el) if el is not None else None)
        return (sp, lp.view(np.complex128) if lp is not None else None,
                el.view(np.complex128) if el is not None else None)


class MonteCarloLoop(_Ensemble):
    """MonteCarloLoop(num_samples, num_sweeps, num_thermalization_sweeps, num_markov_chains, gpu)
    (source/spin_ensembles/MonteCarloLoop.cu:20-42); ``seed`` keys the chains' Philox streams."""

    def __init__(self, num_samples, num_sweeps=1, num_thermalization_sweeps=0, num_markov_chains=1, gpu=True,
                 seed=0):
        h = _handle()
        if isinstance(num_samples, MonteCarloLoop):   # MonteCarloLoop(MonteCarloLoop&)
            call("rbmg_mc_copy", num_samples._h, C.byref(h))
            self.num_markov_chains = num_samples.num_markov_chains
        else:
            call("rbmg_mc_create", int(num_samples), int(num_sweeps), int(num_thermalization_sweeps),
                 int(num_markov_chains), int(seed), C.byref(h))
            self.num_markov_chains = int(num_markov_chains)
        self._h = h

    def set_total_z_symmetry(self, sector):
        call("rbmg_mc_set_total_z_symmetry", self._h, int(sector))

    def set_fast_sweep(self, num_tries):
        call("rbmg_mc_set_fast_sweep", self._h, int(num_tries))

    def acceptance(self, per_chain=False):
        """(accepts, proposals) of the last pass, summed over chains; per_chain=True adds the
        accept counts of every chain (extension: the reference counts globally)."""
        a, p = C.c_uint64(), C.c_uint64()
        if per_chain:
            pc = np.zeros(self.num_markov_chains, np.uint64)
            call("rbmg_mc_acceptance", self._h, C.byref(a), C.byref(p), _p(pc, _u64p))
            return a.value, p.value, pc
        call("rbmg_mc_acceptance", self._h, C.byref(a), C.byref(p), None)
        return a.value, p.value

    @property
    def acceptance_rate(self):
        a, p = self.acceptance()
        return float(a) / float(p) if p else float("nan")


class ExactSummation(_Ensemble):
    """ExactSummation(N, gpu) (source/spin_ensembles/ExactSummation.cu:16-45)."""

    def __init__(self, num_spins, gpu=True):
        h = _handle()
        call("rbmg_exact_create", int(num_spins), C.byref(h))
        self._h = h

    def set_total_z_symmetry(self, sector):
        call("rbmg_exact_set_total_z_symmetry", self._h, int(sector))


class FixedSamples(_Ensemble):
    """Extension: a fixed set of configurations (spins words [count, nwords]), each with
    weight 1 / count, e.g. the samples of an earlier MonteCarloLoop pass
    (`ensemble.samples(psi)`); every estimator accepts it."""

    def __init__(self, num_spins, spins_words):
        w = np.ascontiguousarray(spins_words, np.uint64).reshape(-1, nwords(num_spins))
        h = _handle()
        call("rbmg_samples_create", int(num_spins), len(w), _p(w, _u64p), C.byref(h))
        self._h = h


# --------------------------------------------------------------------- reductions
class ExpectationValue:
    """source/network_functions/ExpectationValue.cu (pyRBMonGPU/main.cpp:295-339)."""

    def __init__(self, gpu=True):
        self.gpu = gpu

    def __call__(self, psi, operator_, spin_ensemble):
        if isinstance(operator_, (list, tuple)):
            ops = (C.c_void_p * len(operator_))(*[o._h for o in operator_])
            out = np.zeros(2 * len(operator_))
            call("rbmg_ev_values", psi._h, ops, len(operator_), spin_ensemble._h, _p(out))
            return list(out.view(np.complex128))
        out = np.zeros(2)
        call("rbmg_ev_value", psi._h, operator_._h, spin_ensemble._h, _p(out))
        return complex(out[0], out[1])

    def fluctuation(self, psi, operator_, spin_ensemble):
        sig = C.c_double()
        out = np.zeros(2)
        call("rbmg_ev_fluctuation", psi._h, operator_._h, spin_ensemble._h, C.byref(sig), _p(out))
        return sig.value, complex(out[0], out[1])

    def gradient(self, psi, operator_, spin_ensemble):
        g = np.zeros(psi.num_params, np.complex128)
        out = np.zeros(2)
        call("rbmg_ev_gradient", psi._h, operator_._h, spin_ensemble._h, _p(g.view(np.float64)), _p(out))
        return g, complex(out[0], out[1])

    def fluctuation_gradient(self, psi, operator_, spin_ensemble):
        """ExpectationValue.cu:258-348 (main.cpp:301, 310): the gradient [P] of the energy
        fluctuation sigma = sqrt(<|E_loc|^2> - |<E_loc>|^2)."""
        g = np.zeros(psi.num_params, np.complex128)
        call("rbmg_ev_fluctuation_gradient", psi._h, operator_._h, spin_ensemble._h, _p(g.view(np.float64)), None)
        return g

    def difference(self, psi, psi_prime, operator_list, spin_ensemble):
        """ExpectationValue.cu:350-446 (main.cpp:304, 323): per operator
        <E'_loc> - <r E_loc> / <r> over psi's ensemble, r = |psi / psi_prime|^2 (Psi only)."""
        ops = (C.c_void_p * len(operator_list))(*[o._h for o in operator_list])
        out = np.zeros(2 * len(operator_list))
        call("rbmg_ev_difference", psi._h, psi_prime._h, ops, len(operator_list), spin_ensemble._h, _p(out))
        return list(out.view(np.complex128))

    def corrected(self, psi, operator_, operator2, spin_ensemble):
        """ExpectationValue.cu:76-127 (main.cpp:309, 328) -> (<E> / <a>, <a>) with
        a = exp(2 Im E + Re(E E - E)); like the reference it evaluates operator_ twice and
        does not use operator2."""
        out = np.zeros(2)
        a = C.c_double()
        call("rbmg_ev_corrected", psi._h, operator_._h, operator2._h, spin_ensemble._h, _p(out), C.byref(a))
        return complex(out[0], out[1]), a.value

    def eloc_gradient(self, psi, operator_, spin_ensemble, score=True):
        """Extension (PsiDeep): the adjoint-kernel gradient, in PyTorch's convention
        dL/dRe + i dL/dIm.  score=False: L = Re <E_loc> on the ensemble's samples held
        fixed; score=True: L = <H> (the sampling term included).  -> (grad[P], <E_loc>)"""
        g = np.zeros(psi.num_params, np.complex128)
        out = np.zeros(2)
        call("rbmg_ev_eloc_gradient", psi._h, operator_._h, spin_ensemble._h, int(bool(score)),
             _p(g.view(np.float64)), _p(out))
        return g, complex(out[0], out[1])


def local_energies(psi, operator_, spins_words):
    """Extension: E_loc of given configurations (uint64 words [count][nwords])."""
    w = np.ascontiguousarray(spins_words, np.uint64).reshape(-1, nwords(psi.N))
    out = np.zeros(2 * len(w))
    call("rbmg_local_energies", psi._h, operator_._h, len(w), _p(w, _u64p), _p(out))
    return out.view(np.complex128)


class HilbertSpaceDistance:
    """source/network_functions/HilbertSpaceDistance.cu (pyRBMonGPU/main.cpp:342-418)."""

    def __init__(self, N, num_params, gpu=True):
        self.N = N
        self.num_params = num_params

    def __call__(self, psi, psi_prime, operator_, is_unitary, spin_ensemble):
        d = C.c_double()
        call("rbmg_hsd_distance", psi._h, psi_prime._h, operator_._h, int(bool(is_unitary)), spin_ensemble._h,
             C.byref(d))
        return d.value

    def distance_2nd_order(self, psi, psi_prime, expr, spin_ensemble, expr_squared=None):
        """distance_2nd_order (pyRBMonGPU/main.cpp:352-363): the reference builds
        Operator(expr) and Operator(expr * expr) from a PauliExpression; here ``expr`` is an
        Operator (or anything Operator accepts) and its square is formed from its Pauli
        tables (``operators.product``) unless given."""
        from . import operators

        def as_op(x):
            if isinstance(x, Operator):
                return x
            return Operator(*x) if isinstance(x, (tuple, list)) else Operator(x)
        op = as_op(expr)
        if expr_squared is None:
            t = (op.coefficients, op.pauli_types, op.pauli_indices)
            expr_squared = Operator(*operators.product(t, t))
        op2 = as_op(expr_squared)
        d = C.c_double()
        call("rbmg_hsd_distance_2nd_order", psi._h, psi_prime._h, op._h, op2._h, spin_ensemble._h, C.byref(d))
        return d.value

    def gradient(self, psi, psi_prime, operator_, is_unitary, spin_ensemble, nu=1.0):
        g = np.zeros(psi_prime.num_params, np.complex128)
        d = C.c_double()
        call("rbmg_hsd_gradient", psi._h, psi_prime._h, operator_._h, int(bool(is_unitary)), spin_ensemble._h,
             C.c_float(nu), _p(g.view(np.float64)), C.byref(d))
        return g, d.value


class KullbackLeibler:
    """KullbackLeibler(num_params, gpu) (pyRBMonGPU/main.cpp:421-470): ``__call__(psi,
    psi_prime, spin_ensemble)`` -> value, ``gradient(psi, psi_prime, spin_ensemble, nu)``
    -> (grad[P], value), with D = log psi' - log psi, value = sqrt(<|D|^2> - |<D>|^2)."""

    def __init__(self, num_params, gpu=True):
        self.num_params = num_params

    def __call__(self, psi, psi_prime, spin_ensemble):
        v = C.c_double()
        call("rbmg_kl_gradient", psi._h, psi_prime._h, spin_ensemble._h, 1.0, None, C.byref(v))
        return v.value

    def gradient(self, psi, psi_prime, spin_ensemble, nu=1.0):
        g = np.zeros(psi_prime.num_params, np.complex128)
        v = C.c_double()
        call("rbmg_kl_gradient", psi._h, psi_prime._h, spin_ensemble._h, float(nu), _p(g.view(np.float64)),
             C.byref(v))
        return g, v.value


class DiagDensityOp:
    """DiagDensityOp(sub_system_size, gpu) (pyRBMonGPU/main.cpp:497-533): called with
    (psi, operator_, spin_ensemble) it returns the 2^sub_system_size densities
    <|E_loc|^2> binned by the configuration of the first sub_system_size spins."""

    def __init__(self, sub_system_size, gpu=True):
        self.sub_system_size = int(sub_system_size)

    def __call__(self, psi, operator_, spin_ensemble):
        out = np.zeros(1 << self.sub_system_size)
        call("rbmg_diag_density", psi._h, operator_._h, spin_ensemble._h, self.sub_system_size, _p(out))
        return out


def psi_O_k_vector(psi, spins):
    """source/network_functions/PsiOkVector.cu:9-44 (entries [0, 2N) are zero)."""
    w = spins_to_words(spins, psi.N)
    out = np.zeros(psi.num_params, np.complex128)
    call("rbmg_psi_O_k_vector", psi._h, _p(w, _u64p), _p(out.view(np.float64)))
    return out


def get_S_matrix(psi, spin_ensemble, weighted=False, centered=False, simt=False):
    """get_S_matrix (source/network_functions/S_matrix.cu:10-53; C++ only in the
    reference): S[k, k'] = sum_s O_k(s) conj(O_k'(s)) / num_steps over the ensemble's
    configurations, P x P complex128 with zero rows and columns below 2N.  As in the
    reference the exact-summation weight is not applied; ``weighted=True`` applies the
    normalised |psi|^2, ``centered=True`` subtracts <O_k> conj(<O_k'>).  The products run
    on the tensor cores; ``simt=True`` takes the FP32 CUDA-core kernel instead."""
    P = psi.num_params
    out = np.zeros((P, P), np.complex128)
    flags = (1 if weighted else 0) | (2 if centered else 0) | (4 if simt else 0)
    call("rbmg_s_matrix", psi._h, spin_ensemble._h, flags, _p(out.view(np.float64)))
    return out


# --------------------------------------------------------------------- persistent chains
class Chain:
    """Walkers whose configurations and Philox positions stay on the device between
    calls (extension: the reference's foreach restarts its chains every call)."""

    def __init__(self, psi, num_walkers, seed=0):
        h = _handle()
        call("rbmg_chain_create", psi._h, int(num_walkers), int(seed), C.byref(h))
        self._h = h
        self.num_walkers = int(num_walkers)
        self.N = psi.N
        self._host = None

    def __del__(self):
        h, self._h = getattr(self, "_h", None), None
        if h is not None:
            try:
                lib().rbmg_chain_destroy(h)
            except Exception:
                pass

    def sweep_async(self, psi, operator_=None, n_sweeps=1, measure_every=1, d_eloc=0, stream=None):
        """Device-level call: d_eloc is a device address of double2 [n_sweeps // measure_every][walkers]."""
        call("rbmg_chain_sweep_async", self._h, psi._h, operator_._h if operator_ is not None else None,
             int(n_sweeps), int(measure_every), C.c_void_p(d_eloc) if d_eloc else None,
             C.c_void_p(stream) if stream else None)

    def set_learned_streams(self, streams):
        """Frozen learned steps on 1 to 4 streams (0: automatic, 2 from 8192 walkers on)."""
        call("rbmg_chain_set_learned_streams", self._h, int(streams))

    def learned_async(self, psi, operator_, proposal, n_steps, train=0, measure_every=1, d_eloc=0, stream=None):
        """n_steps learned Metropolis-Hastings steps (cluster flips picked by `proposal`).
        train > 0: one REINFORCE + Adam update per step on the first `train` walkers' moves;
        train = 0: frozen proposal, exactly |psi|^2-stationary.  d_eloc: device address of
        double2 [n_steps // measure_every][walkers], or 0."""
        call("rbmg_chain_learned_async", self._h, psi._h, operator_._h if operator_ is not None else None,
             proposal._h, int(n_steps), int(train), int(measure_every), C.c_void_p(d_eloc) if d_eloc else None,
             C.c_void_p(stream) if stream else None)

    def learned_kernel_times(self, psi, proposal, n_steps):
        """Measurement hook: mean (network pass, accept pass) durations in ms over n_steps
        frozen learned steps on one stream."""
        a, b = C.c_double(), C.c_double()
        call("rbmg_chain_learned_kernel_times", self._h, psi._h, proposal._h, int(n_steps), C.byref(a), C.byref(b))
        return a.value, b.value

    def learned_trace(self, psi, proposal, n_steps):
        """Test hook: n_steps frozen learned steps with the state recorded around every
        launch (rbmg_chain_learned_trace); returns a dict of host arrays."""
        B, N, nw = self.num_walkers, self.N, nwords(self.N)
        Mpad = (psi.M + 31) // 32 * 32
        O = N + Proposal.LENGTHS
        f32 = lambda *sh: np.zeros(sh, np.float32)   # noqa: E731
        d = dict(spins0=np.zeros((B, nw), np.uint64), rng0=np.zeros(B, np.uint64), theta0=f32(B, Mpad, 2),
                 re0=f32(B, Mpad), logits0=f32(B, O), logits_prop=f32(n_steps, B, O),
                 site=np.zeros((n_steps, B), np.int32), len=np.zeros((n_steps, B), np.int32),
                 logq=f32(n_steps, B), spins=np.zeros((n_steps, B, nw), np.uint64),
                 accepts=np.zeros((n_steps, B), np.uint64), rng_end=np.zeros(B, np.uint64))
        fp = C.POINTER(C.c_float)
        ip = C.POINTER(C.c_int)
        call("rbmg_chain_learned_trace", self._h, psi._h, proposal._h, int(n_steps), _p(d["spins0"], _u64p),
             _p(d["rng0"], _u64p), _p(d["theta0"], fp), _p(d["re0"], fp), _p(d["logits0"], fp),
             _p(d["logits_prop"], fp), _p(d["site"], ip), _p(d["len"], ip), _p(d["logq"], fp),
             _p(d["spins"], _u64p), _p(d["accepts"], _u64p), _p(d["rng_end"], _u64p))
        return d

    def checkpoint(self):
        """{spins, rng_index, accepts, proposals}: restoring it continues the chains bit for bit."""
        B = self.num_walkers
        d = dict(spins=np.zeros((B, nwords(self.N)), np.uint64), rng_index=np.zeros(B, np.uint64),
                 accepts=np.zeros(B, np.uint64), proposals=np.zeros(B, np.uint64))
        call("rbmg_chain_get_checkpoint", self._h, *[_p(d[k], _u64p) for k in ("spins", "rng_index", "accepts",
                                                                              "proposals")])
        return d

    def restore(self, ckpt):
        d = {k: np.ascontiguousarray(ckpt[k], np.uint64) for k in ("spins", "rng_index", "accepts", "proposals")}
        call("rbmg_chain_set_checkpoint", self._h, *[_p(d[k], _u64p) for k in ("spins", "rng_index", "accepts",
                                                                              "proposals")])

    def save(self, path):
        np.savez(path, **self.checkpoint())

    def load(self, path):
        with np.load(path) as f:
            self.restore({k: f[k] for k in f.files})

    def state(self):
        sp = np.zeros((self.num_walkers, nwords(self.N)), np.uint64)
        a, p = C.c_uint64(), C.c_uint64()
        call("rbmg_chain_state", self._h, _p(sp, _u64p), C.byref(a), C.byref(p))
        return sp, a.value, p.value


class Proposal:
    """Learned cluster-flip proposal (extension): an MLP N -> 256 -> 256 (SiLU) -> N seed +
    8 length logits with BF16 operands and FP32 accumulation, trained by the chain
    (Chain.learned_async).  Parameters are FP32 in the order W1 [N][256], b1, W2 [256][256],
    b2, W3 [256][N+8], b3."""

    HIDDEN = 256
    LENGTHS = 8
    LOCALLY_BALANCED = 0
    REINFORCE = 1

    def __init__(self, N, seed=0, lr=1e-3, objective=LOCALLY_BALANCED):
        h = _handle()
        call("rbmg_proposal_create", int(N), int(seed), float(lr), C.byref(h))
        self._h = h
        self.N = int(N)
        n = C.c_int64()
        call("rbmg_proposal_num_params", h, C.byref(n))
        self.num_params = n.value
        self.set_objective(objective)

    def set_objective(self, objective):
        """LOCALLY_BALANCED (default): cross-entropy to p*(i, l) propto |psi(s')/psi(s)| over
        all cluster moves; REINFORCE: policy gradient on the acceptance."""
        call("rbmg_proposal_set_objective", self._h, int(objective))

    def __del__(self):
        h, self._h = getattr(self, "_h", None), None
        if h is not None:
            try:
                lib().rbmg_proposal_destroy(h)
            except Exception:
                pass

    @property
    def params(self):
        out = np.zeros(self.num_params, np.float32)
        call("rbmg_proposal_get_params", self._h, _p(out, C.POINTER(C.c_float)))
        return out

    @params.setter
    def params(self, v):
        v = np.ascontiguousarray(v, np.float32)
        if v.shape != (self.num_params,):
            raise ValueError(f"expected {self.num_params} parameters")
        call("rbmg_proposal_set_params", self._h, _p(v, C.POINTER(C.c_float)))

    def eval(self, spins, dlogits=None):
        """Forward pass on configurations (uint64 words [count][nwords]) -> logits
        [count][N+8]; with dlogits also the parameter gradient of sum(dlogits * logits)."""
        sp = np.ascontiguousarray(spins, np.uint64).reshape(-1, nwords(self.N))
        count = sp.shape[0]
        logits = np.zeros((count, self.N + self.LENGTHS), np.float32)
        fp = C.POINTER(C.c_float)
        if dlogits is None:
            call("rbmg_proposal_eval", self._h, count, _p(sp, _u64p), None, _p(logits, fp), None)
            return logits
        dl = np.ascontiguousarray(dlogits, np.float32).reshape(count, self.N + self.LENGTHS)
        grads = np.zeros(self.num_params, np.float32)
        call("rbmg_proposal_eval", self._h, count, _p(sp, _u64p), _p(dl, fp), _p(logits, fp), _p(grads, fp))
        return logits, grads

    def lb_target(self, psi, spins, logits):
        """Test hook: the locally balanced training target (q - p*) / count of the
        configurations `spins` (uint64 words [count][nwords]) under `logits` [count][N+8]."""
        sp = np.ascontiguousarray(spins, np.uint64).reshape(-1, nwords(self.N))
        lg = np.ascontiguousarray(logits, np.float32).reshape(len(sp), self.N + self.LENGTHS)
        dl = np.zeros_like(lg)
        fp = C.POINTER(C.c_float)
        call("rbmg_proposal_lb_target", self._h, psi._h, len(sp), _p(sp, _u64p), _p(lg, fp), _p(dl, fp))
        return dl

    def checkpoint(self):
        """{params, m, v, steps}: the network and its Adam state."""
        fp = C.POINTER(C.c_float)
        d = dict(params=np.zeros(self.num_params, np.float32), m=np.zeros(self.num_params, np.float32),
                 v=np.zeros(self.num_params, np.float32))
        steps = C.c_int64()
        call("rbmg_proposal_get_state", self._h, _p(d["params"], fp), _p(d["m"], fp), _p(d["v"], fp),
             C.byref(steps))
        d["steps"] = steps.value
        return d

    def restore(self, ckpt):
        fp = C.POINTER(C.c_float)
        arr = {k: np.ascontiguousarray(ckpt[k], np.float32) for k in ("params", "m", "v")}
        call("rbmg_proposal_set_state", self._h, _p(arr["params"], fp), _p(arr["m"], fp), _p(arr["v"], fp),
             int(ckpt["steps"]))

    def status(self):
        """Waits for the device; raises if a tensor-core pass of the network timed out."""
        call("rbmg_proposal_status", self._h)

    def adam(self, grads):
        """One Adam step (betas 0.9 / 0.999, eps 1e-8) with the given gradient."""
        g = np.ascontiguousarray(grads, np.float32)
        call("rbmg_proposal_adam", self._h, _p(g, C.POINTER(C.c_float)))


class Batch:
    """Many complex RBMs of uneven N and M served by one persistent launch replayed from a
    CUDA graph (extension).  instances: list of (psi, operator, walkers, seed)."""

    def __init__(self, instances):
        self._keep = [(p, o) for p, o, _, _ in instances]
        n = len(instances)
        psis = (C.c_void_p * n)(*[p._h.value for p, _, _, _ in instances])
        ops = (C.c_void_p * n)(*[o._h.value for _, o, _, _ in instances])
        walkers = (C.c_uint32 * n)(*[int(w) for _, _, w, _ in instances])
        seeds = (C.c_uint64 * n)(*[int(sd) for _, _, _, sd in instances])
        h = _handle()
        call("rbmg_batch_create", n, psis, ops, walkers, seeds, C.byref(h))
        self._h = h
        self.instances = [(p.N, p.num_params, int(w)) for p, _, w, _ in instances]

    def __del__(self):
        h, self._h = getattr(self, "_h", None), None
        if h is not None:
            try:
                lib().rbmg_batch_destroy(h)
            except Exception:
                pass

    def run(self, therm=0, sweeps=1):
        call("rbmg_batch_run", self._h, int(therm), int(sweeps))

    def set_shape(self, warps_per_block, rows):
        call("rbmg_batch_set_shape", self._h, int(warps_per_block), int(rows))

    @property
    def shape(self):
        w, r, b = C.c_int(), C.c_int(), C.c_int()
        call("rbmg_batch_get_shape", self._h, C.byref(w), C.byref(r), C.byref(b))
        return w.value, r.value, b.value

    def set_wait(self, seconds=20.0, extra_walkers=0):
        """Wall-clock limit of a reduction task's wait for its instance's walkers; with
        extra_walkers > 0 the wait cannot end and runs out (the bounded-wait test)."""
        call("rbmg_batch_set_wait", self._h, float(seconds), int(extra_walkers))

    @property
    def register_cap(self):
        r = C.c_int()
        call("rbmg_batch_get_register_cap", self._h, C.byref(r))
        return r.value

    @register_cap.setter
    def register_cap(self, regs):
        call("rbmg_batch_set_register_cap", self._h, int(regs))

    def autotune(self, sweeps=1, reps=3):
        """Times the launch shapes on the batch itself, keeps the fastest; returns
        {(register_cap, warps_per_block, rows): ms per replay}."""
        ms = np.zeros(18)
        call("rbmg_batch_autotune", self._h, int(sweeps), int(reps), _p(ms))
        shapes = [(c, w, r) for c in (255, 128, 96) for w in (2, 4, 8) for r in (8, 16)]
        return dict(zip(shapes, ms.tolist()))

    def result(self, i, want_eloc=False):
        """(<E_loc>, O_k gradient [P], local energies or None) of instance i, last replay: the
        reference's estimator <E O*> + conj<E_k> - 2 <E> <O*> over its walkers."""
        N, P, w = self.instances[i]
        e = np.zeros(2)
        g = np.zeros(P, np.complex128)
        el = np.zeros(w, np.complex128) if want_eloc else None
        call("rbmg_batch_result", self._h, int(i), _p(e), _p(g.view(np.float64)),
             _p(el.view(np.float64)) if want_eloc else None)
        return complex(e[0], e[1]), g, el

    def spins(self, i):
        """The configurations of instance i's walkers after the last replay (uint64 words)."""
        N, _, w = self.instances[i]
        sp = np.zeros((w, nwords(N)), np.uint64)
        call("rbmg_batch_spins", self._h, int(i), _p(sp, _u64p))
        return sp

    def accepts(self):
        a = C.c_uint64()
        call("rbmg_batch_info", self._h, None, C.byref(a), None)
        return a.value


def library_stream():
    """The library's CUDA stream of the calling thread (a cudaStream_t as int)."""
    st = C.c_void_p()
    call("rbmg_stream", C.byref(st))
    return st.value or 0


# --------------------------------------------------------------------- factories
def real_noise(shape, rng=np.random):
    return 2 * rng.random_sample(shape) - 1


def complex_noise(shape, rng=np.random):
    return real_noise(shape, rng) + 1j * real_noise(shape, rng)


def new_neural_network(N, M, initial_value=(0.01 + 1j * math.pi / 4), alpha=0, beta=0, free_quantum_axis=False,
                       noise=1e-6, gpu=True):
    """pyRBMonGPU/new_neural_network.py:29-50"""
    if isinstance(alpha, (int, float)):
        alpha = alpha * np.ones(N)
    if isinstance(beta, (int, float)):
        beta = beta * np.ones(N)
    b = noise * complex_noise(M)
    W = noise * complex_noise((N, M))
    for r in range(M // N):
        W[:, r * N:(r + 1) * N] += initial_value * np.diag(np.ones(N))
    return Psi(alpha, beta, b, W, 1, free_quantum_axis, gpu)


def new_deep_neural_network(N, M, C_, initial_value=(0.01 + 1j * math.pi / 4), alpha=0, beta=0,
                            free_quantum_axis=False, noise=1e-4, gpu=True, pair=False, noise_modulation="auto",
                            final_weights=10):
    """pyRBMonGPU/new_neural_network.py:53-153.  1D: N spins, layer sizes M [l], connections
    per unit C_ [l].  2D: N = (rows, cols), M and C_ lists of (rows, cols) pairs; unit (j1, j2)
    of a layer connects to the units ((j1 d1 + i1) % n0, (j2 d2 + i2) % n1) of the layer below,
    numbered row * n0 + col as the reference numbers them.  numpy's global random state is
    consumed in the reference's order, so a seeded caller gets the reference's network."""
    dim = len(N) if isinstance(N, (list, tuple)) else 1
    N_lin = N if dim == 1 else N[0] * N[1]
    M_lin = M if dim == 1 else [m[0] * m[1] for m in M]
    C_lin = C_ if dim == 1 else [c[0] * c[1] for c in C_]
    for n, m, c in zip([N] + M[:-1], M, C_):
        if dim == 1:
            assert (m * c) % n == 0
            assert c <= n
        else:
            assert (m[0] * c[0]) % n[0] == 0 and (m[1] * c[1]) % n[1] == 0
            assert c[0] <= n[0] and c[1] <= n[1]
    if isinstance(alpha, (float, int)):
        alpha = alpha * np.ones(N_lin)
    if isinstance(beta, (float, int)):
        beta = beta * np.ones(N_lin)
    b = [noise * complex_noise(m) for m in M_lin]
    w = noise * complex_noise((C_lin[0], M_lin[0]))
    w[C_lin[0] // 2, :] += initial_value
    W = [w]
    if noise_modulation == "auto":
        noise_modulation = [math.sqrt(6 / (c + next_c)) for c, next_c in zip(C_lin[1:], C_lin[2:] + [1])]
    for c, m, next_c, nm in zip(C_lin[1:], M_lin[1:], C_lin[2:] + [1], noise_modulation):
        W.append(nm * math.sqrt(6 / (c + next_c)) * real_noise((c, m)) + noise * complex_noise((c, m)))

    def delta_func(n, m, c):
        if m > n:
            return 1
        if n % m == 0:
            return n // m
        return c

    connections = []
    for n, m, c in zip([N] + M[:-1], M, C_):
        if dim == 1:
            d = delta_func(n, m, c)
            connections.append(np.array([[(j * d + i) % n for j in range(m)] for i in range(c)]))
        else:
            d1, d2 = delta_func(n[0], m[0], c[0]), delta_func(n[1], m[1], c[1])
            units = [(j1, j2) for j1 in range(m[0]) for j2 in range(m[1])]
            inputs = [(i1, i2) for i1 in range(c[0]) for i2 in range(c[1])]
            connections.append(np.array([[((j1 * d1 + i1) % n[0]) * n[0] + (j2 * d2 + i2) % n[1]
                                          for j1, j2 in units] for i1, i2 in inputs]))
    if isinstance(final_weights, (float, int)):
        final_weights = final_weights * np.ones(M_lin[-1])
    assert len(final_weights) == M_lin[-1]
    cls = PsiPair if pair else PsiDeep
    return cls(alpha, beta, b, connections, W, final_weights, 1.0, free_quantum_axis, gpu)


__all__ = ["Batch", "Chain", "library_stream", "Psi", "PsiDeep", "PsiPair", "Operator", "Spins", "MonteCarloLoop", "ExactSummation",
           "ExpectationValue", "HilbertSpaceDistance", "psi_O_k_vector", "activation_function", "setDevice",
           "start_profiling", "stop_profiling", "new_neural_network", "new_deep_neural_network", "RbmgError"]
