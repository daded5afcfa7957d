/*
 * CPU restatement ("oracle") of RBMonGPU's variational hot path.
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/, the smoke check and the benchmark's
 * CPU-baseline leg as the checker of the CUDA kernels; never linked into the
 * product library.  Build: oracle/Makefile (gcc -O2 -ffp-contract=off).
 *
 * Every function cites the reference file:line it restates (paths relative to the
 * RBMonGPU source tree).
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------- */
/* small complex helpers (FP64)                                              */
/* ------------------------------------------------------------------------- */
typedef struct { double re, im; } cd;

static inline cd C(double re, double im) { cd z = {re, im}; return z; }
static inline cd cadd(cd a, cd b) { return C(a.re + b.re, a.im + b.im); }
static inline cd csub(cd a, cd b) { return C(a.re - b.re, a.im - b.im); }
static inline cd cmul(cd a, cd b) { return C(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
static inline cd cscale(double s, cd a) { return C(s * a.re, s * a.im); }
static inline cd cconj(cd a) { return C(a.re, -a.im); }
static inline cd cdiv(cd a, cd b) {
    const double den = b.re * b.re + b.im * b.im;
    return C((a.re * b.re + a.im * b.im) / den, (a.im * b.re - a.re * b.im) / den);
}
static inline cd cexp_(cd a) {
    const double e = exp(a.re);
    return C(e * cos(a.im), e * sin(a.im));
}
static inline double cnorm(cd a) { return a.re * a.re + a.im * a.im; }
static inline cd cload(const double* p, long i) { return C(p[2 * i], p[2 * i + 1]); }
static inline void cstore(double* p, long i, cd z) { p[2 * i] = z.re; p[2 * i + 1] = z.im; }
static inline void cacc(double* p, long i, cd z) { p[2 * i] += z.re; p[2 * i + 1] += z.im; }

/* ------------------------------------------------------------------------- */
/* spins (include/Spins.h:32-217)                                            */
/* ------------------------------------------------------------------------- */
static inline int nwords_of(int N) { return (N + 63) / 64; }
static inline double spin_at(const uint64_t* s, int i) {           /* Spins.h:125-129 */
    return ((s[i >> 6] >> (i & 63)) & 1u) ? 1.0 : -1.0;
}
static inline void spin_flip(uint64_t* s, int i) { s[i >> 6] ^= (uint64_t)1 << (i & 63); }
static inline void spins_mask(uint64_t* s, int N) {                 /* Spins.h:98-101 */
    const int w = N / 64;
    if (w < nwords_of(N)) s[w] &= ((uint64_t)1 << (N % 64)) - 1u;
}
static inline int spins_equal(const uint64_t* a, const uint64_t* b, int nw) {
    for (int k = 0; k < nw; k++) if (a[k] != b[k]) return 0;
    return 1;
}

/* ------------------------------------------------------------------------- */
/* random streams                                                            */
/* ------------------------------------------------------------------------- */

/* Philox4x32-10, Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as
 * 1, 2, 3" (SC'11): ten rounds of two 32x32->64 multiplies with a Weyl key schedule. */
void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; r++) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Walker stream: word `index` of walker `walker` = component index%4 of the block
 * counter (index/4 lo, index/4 hi, walker, 0x52424D47) under key (seed lo, seed hi). */
uint32_t or_philox_word(uint64_t seed, uint32_t walker, uint64_t index) {
    const uint64_t block = index >> 2;
    const uint32_t ctr[4] = {(uint32_t)block, (uint32_t)(block >> 32), walker, 0x52424D47u};
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t out[4];
    or_philox4x32_10(ctr, key, out);
    return out[index & 3];
}

/* MT19937, Matsumoto & Nishimura (1998): the engine the reference's host path uses
 * (std::mt19937(i), source/spin_ensembles/MonteCarloLoop.cu:89-92). */
typedef struct { uint32_t mt[624]; int idx; } mt19937;

static void mt_seed(mt19937* g, uint32_t seed) {
    g->mt[0] = seed;
    for (int i = 1; i < 624; i++)
        g->mt[i] = 1812433253u * (g->mt[i - 1] ^ (g->mt[i - 1] >> 30)) + (uint32_t)i;
    g->idx = 624;
}

static uint32_t mt_next(mt19937* g) {
    if (g->idx >= 624) {
        for (int i = 0; i < 624; i++) {
            const uint32_t y = (g->mt[i] & 0x80000000u) | (g->mt[(i + 1) % 624] & 0x7fffffffu);
            g->mt[i] = g->mt[(i + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908B0DFu : 0u);
        }
        g->idx = 0;
    }
    uint32_t y = g->mt[g->idx++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9D2C5680u;
    y ^= (y << 15) & 0xEFC60000u;
    y ^= y >> 18;
    return y;
}

void or_mt_words(uint32_t seed, int count, uint32_t* out) {
    mt19937 g;
    mt_seed(&g, seed);
    for (int i = 0; i < count; i++) out[i] = mt_next(&g);
}

/* One stream per chain, consumed exactly in the reference's draw order. */
typedef struct {
    int kind;
    mt19937 mt;
    uint64_t seed;
    uint32_t walker;
    uint64_t index;
} rng_t;

/* include/random.h:21-28: uniform_int_distribution<uint64>(0, 2^32-1) over a 32-bit
 * engine returns the raw engine word. */
static uint32_t rng_u32(rng_t* r) {
    if (r->kind == OR_RNG_MT19937) return mt_next(&r->mt);
    return or_philox_word(r->seed, r->walker, r->index++);
}

/* include/random.h:47-54.  Host: uniform_real_distribution<double>(0,1) =
 * generate_canonical<double,53> with two engine words, value in [0,1).
 * Philox stream: ((w >> 8) + 1) * 2^-24, a float in (0,1] like curand_uniform. */
static double rng_real(rng_t* r) {
    if (r->kind == OR_RNG_MT19937) {
        const double x1 = (double)mt_next(&r->mt);
        const double x2 = (double)mt_next(&r->mt);
        double sum = x1;
        sum += x2 * 4294967296.0;
        double ret = sum / 18446744073709551616.0;
        if (ret >= 1.0) ret = nextafter(1.0, 0.0);
        return ret;
    }
    const uint32_t w = rng_u32(r);
    return (double)((float)((w >> 8) + 1u) * 5.9604644775390625e-8f);
}

/* include/Spins.h:87-104 with include/random.h:30-34: one 64-bit word per spin word,
 * low 32 bits drawn first. */
static void rng_spins(rng_t* r, int N, uint64_t* s) {
    const int nw = nwords_of(N);
    for (int k = 0; k < nw; k++) {
        const uint64_t lo = rng_u32(r);
        const uint64_t hi = rng_u32(r);
        s[k] = lo | (hi << 32);
    }
    spins_mask(s, N);
}

/* include/random.h:60-79.  The reference shifts an int (valid for n < 32); the same
 * steps with 64-bit masks, identical for n < 32 and defined up to n = 64. */
static uint64_t rng_n_over_k(rng_t* r, unsigned n, unsigned k) {
    const uint64_t mask = n >= 64 ? ~(uint64_t)0 : (((uint64_t)1 << n) - 1u);
    uint64_t w = rng_u32(r);
    w |= (uint64_t)rng_u32(r) << 32;
    uint64_t result = w & mask;
    int diff = (int)k - (int)__builtin_popcountll(result);
    while (diff != 0) {
        uint64_t w2 = rng_u32(r);
        w2 |= (uint64_t)rng_u32(r) << 32;
        unsigned pos = (unsigned)(w2 % n);
        while (((result >> pos) & 1u) == (uint64_t)(diff > 0)) pos = (pos + 1) % n;
        result ^= (uint64_t)1 << pos;
        if (diff > 0) diff--; else diff++;
    }
    return result;
}

/* ------------------------------------------------------------------------- */
/* activation (include/quantum_state/psi_functions.hpp:49-57, 97-114)        */
/* ------------------------------------------------------------------------- */
static cd lc64(cd z) {
    const double sign = z.re > 0.0 ? 1.0 : -1.0;
    cd t = C(sign * 3.746646023906276 + z.re, z.im);
    t = cmul(z, t); t.re += 7.771429504240965;
    t = cmul(z, t); t.re += sign * 10.2180213465;
    t = cmul(z, t); t.re += 9.19376335670885;
    const cd num = C(5.49914721954 - sign * 2.16564366435 * z.re, -sign * 2.16564366435 * z.im);
    cd res = cadd(cscale(sign * 0.9003320053750442, z), cdiv(num, t));
    res.re -= 0.598139;
    return res;
}

static cd tanh64(cd z) {
    const double sign = z.re > 0.0 ? 1.0 : -1.0;
    cd d = C(sign * 3.746646023906276 + z.re, z.im);
    d = cmul(z, d); d.re += 7.771429504240965;
    d = cmul(z, d); d.re += sign * 10.218021346543315;
    d = cmul(z, d); d.re += 9.19376335670885;
    cd p = C(6.746450656267947 + sign * 0.9003320053750442 * z.re, sign * 0.9003320053750442 * z.im);
    p = cmul(z, p); p.re += sign * 26.632014683761202;
    p = cmul(z, p); p.re += 70.82878897882324;
    p = cmul(z, p); p.re += sign * 146.36284300074402;
    p = cmul(z, p); p.re += 199.24474920889975;
    p = cmul(z, p); p.re += sign * 177.6769746361748;
    p = cmul(z, p); p.re += 83.68563506532087;
    p = cmul(z, p);
    return cdiv(p, cmul(d, d));
}

void or_logcosh(double re, double im, double* out) { cd r = lc64(C(re, im)); out[0] = r.re; out[1] = r.im; }
void or_tanh(double re, double im, double* out) { cd r = tanh64(C(re, im)); out[0] = r.re; out[1] = r.im; }

/* Real activation of PsiPair's real nets (psi_functions.hpp:118-136). */
static inline double relu64(double x) { return x > 0.0 ? x : 0.0; }

/* ---- FP32 operation order of the CUDA sampler (rbmongpu_gb300/csrc/activation.cuh).
 * my_logcosh is even: f(z) = g(u) with u = sign(Re z) * z, so the sign is folded into u
 * and g is evaluated with fixed positive coefficients. ---- */
#define F_LC_A 0.9003320053750442f
#define F_LC_NA 5.49914721954f
#define F_LC_NB 2.16564366435f
#define F_LC_D0 9.19376335670885f
#define F_LC_D1 10.2180213465f
#define F_LC_D2 7.771429504240965f
#define F_LC_D3 3.746646023906276f
#define F_LC_C 0.598139f

typedef struct { float dr, di, p, q; } lc_den32;

static inline lc_den32 lc_den_f32(float x, float y) {
    const float s = x > 0.0f ? 1.0f : -1.0f;
    const float p = s * x, q = s * y;
    const float t1r = p + F_LC_D3;
    const float t2r = fmaf(p, t1r, fmaf(-q, q, F_LC_D2));
    const float t2i = fmaf(p, q, q * t1r);
    const float t3r = fmaf(p, t2r, fmaf(-q, t2i, F_LC_D1));
    const float t3i = fmaf(p, t2i, q * t2r);
    lc_den32 d;
    d.dr = fmaf(p, t3r, fmaf(-q, t3i, F_LC_D0));
    d.di = fmaf(p, t3i, q * t3r);
    d.p = p; d.q = q;
    return d;
}

/* num / den by FMAs (device_math.cuh::div_pos): integer reciprocal estimate
 * 0x7EF311C2 - bits(den), two Newton steps, one residual correction of the quotient */
static inline float div_pos_f32(float num, float den) {
    union { uint32_t u; float f; } b;
    b.f = den;
    b.u = 0x7EF311C2u - b.u;
    float r = b.f;
    r = fmaf(r, fmaf(-den, r, 1.0f), r);
    r = fmaf(r, fmaf(-den, r, 1.0f), r);
    const float q = num * r;
    return fmaf(r, fmaf(-den, q, num), q);
}

/* div_pos_f32 over arrays (a test hook: the reciprocal's error bound) */
void or_div_pos_f32_n(const float* num, const float* den, float* out, long n) {
    for (long i = 0; i < n; i++) out[i] = div_pos_f32(num[i], den[i]);
}

float or_lc_re_f32(float x, float y) {
    const lc_den32 d = lc_den_f32(x, y);
    const float nr = fmaf(-F_LC_NB, d.p, F_LC_NA);
    const float ni = -F_LC_NB * d.q;
    const float num = fmaf(nr, d.dr, ni * d.di);
    const float den = fmaf(d.dr, d.dr, d.di * d.di);
    return fmaf(F_LC_A, d.p, div_pos_f32(num, den)) - F_LC_C;
}

void or_lc_f32(float x, float y, float* out) {
    const lc_den32 d = lc_den_f32(x, y);
    const float nr = fmaf(-F_LC_NB, d.p, F_LC_NA);
    const float ni = -F_LC_NB * d.q;
    const float num_r = fmaf(nr, d.dr, ni * d.di);
    const float num_i = fmaf(ni, d.dr, -(nr * d.di));
    const float den = fmaf(d.dr, d.dr, d.di * d.di);
    out[0] = fmaf(F_LC_A, d.p, num_r / den) - F_LC_C;
    out[1] = fmaf(F_LC_A, d.q, num_i / den);
}

void or_tanh_f32(float x, float y, float* out) {
    double r[2];
    or_tanh((double)x, (double)y, r);
    out[0] = (float)r[0];
    out[1] = (float)r[1];
}

/* Deterministic expf: Cody & Waite (1980) two-constant range reduction x = n ln2 + r,
 * |r| <= ln2/2, then the degree-7 Taylor polynomial of e^r in Horner form and an exact
 * power-of-two scale.  Only fmaf/mul/add are used, so CPU and GPU round identically. */
float or_expf_det(float x) {
    if (x < -87.0f) return 0.0f;
    if (x > 88.0f) x = 88.0f;
    const float n = rintf(x * 1.44269502f);
    float r = fmaf(n, -0.693145752f, x);
    r = fmaf(n, -1.42860677e-06f, r);
    float p = 1.98412698e-04f;
    p = fmaf(p, r, 1.38888889e-03f);
    p = fmaf(p, r, 8.33333333e-03f);
    p = fmaf(p, r, 4.16666667e-02f);
    p = fmaf(p, r, 1.66666667e-01f);
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    const int e = (int)n;
    /* 2^e split in two factors so that e down to -126-ish stays normal */
    const int e1 = e / 2, e2 = e - e / 2;
    union { uint32_t u; float f; } s1, s2;
    s1.u = (uint32_t)(e1 + 127) << 23;
    s2.u = (uint32_t)(e2 + 127) << 23;
    return (p * s1.f) * s2.f;
}

/* Deterministic log of a positive normal float, the operation order of
 * rbmongpu_gb300/csrc/device_math.cuh::logf_det: x = 2^e m, m in [sqrt(1/2), sqrt(2)),
 * log m = 2 atanh(t), t = (m - 1)/(m + 1), by the odd series to t^13 (Horner in t^2),
 * plus e ln2 in Cody & Waite's two constants. */
float or_logf_det(float x) {
    union { uint32_t u; float f; } b;
    b.f = x;
    int e = (int)((b.u >> 23) & 0xffu) - 127;
    b.u = (b.u & 0x007fffffu) | 0x3f800000u;
    float m = b.f;
    if (m > 1.41421356f) { m = m * 0.5f; e += 1; }
    const float t = (m + -1.0f) / (m + 1.0f);
    const float t2 = t * t;
    float p = 7.69230769e-02f;
    p = fmaf(p, t2, 9.09090909e-02f);
    p = fmaf(p, t2, 1.11111111e-01f);
    p = fmaf(p, t2, 1.42857143e-01f);
    p = fmaf(p, t2, 2.00000000e-01f);
    p = fmaf(p, t2, 3.33333333e-01f);
    p = fmaf(p, t2, 1.0f);
    const float lm = (2.0f * t) * p;
    const float ef = (float)e;
    return ef * 0.693145752f + fmaf(ef, 1.42860677e-06f, lm);
}

/* ------------------------------------------------------------------------- */
/* RBM (include/quantum_state/Psi.hpp:43-202)                                */
/* ------------------------------------------------------------------------- */
static cd rbm_angle(const or_psi* psi, int j, const uint64_t* s) {    /* Psi.hpp:43-53 */
    cd r = cload(psi->b, j);
    for (int i = 0; i < psi->N; i++)
        r = cadd(r, cscale(spin_at(s, i), cload(psi->W, (long)i * psi->M + j)));
    return r;
}

void or_rbm_angles(const or_psi* psi, const uint64_t* spins, double* theta) {
    for (int j = 0; j < psi->M; j++) cstore(theta, j, rbm_angle(psi, j, spins));
}

/* ------------------------------------------------------------------------- */
/* PsiDeep / PsiPair forward pass (include/quantum_state/PsiDeep.hpp:89-169) */
/* ------------------------------------------------------------------------- */
#define DEEP_MAX_UNITS 4096

typedef struct {
    cd angle[OR_MAX_LAYERS][DEEP_MAX_UNITS];
    cd act[OR_MAX_LAYERS + 1][DEEP_MAX_UNITS];   /* act[0] = spins, act[l+1] = activation of layer l */
} deep_cache;

/* part: 0 complex net (kind 1); 1 real part net / 2 imaginary part net (kind 2) */
static void deep_weights(const or_psi* psi, int part, int l, const double** w, const double** bias) {
    if (part == 2) { *w = psi->lhs_w_im[l]; *bias = psi->bias_im[l]; }
    else { *w = psi->lhs_w[l]; *bias = psi->bias[l]; }
}

static cd deep_forward(const or_psi* psi, int part, const uint64_t* s, deep_cache* c) {
    const int is_real = psi->kind == OR_PSI_PAIR;
    for (int i = 0; i < psi->N; i++) c->act[0][i] = C(spin_at(s, i), 0.0);
    for (int l = 0; l < psi->num_layers; l++) {
        const double *w, *bias;
        deep_weights(psi, part, l, &w, &bias);
        const int size = psi->size[l], conn = psi->conn[l];
        for (int j = 0; j < size; j++) {
            cd a = C(0.0, 0.0);
            for (int i = 0; i < conn; i++) {
                const unsigned src = psi->lhs_conn[l][(long)i * size + j];
                const cd wij = is_real ? C(w[(long)i * size + j], 0.0) : cload(w, (long)i * size + j);
                a = cadd(a, cmul(wij, c->act[l][src]));
            }
            a = cadd(a, is_real ? C(bias[j], 0.0) : cload(bias, j));
            c->angle[l][j] = a;
        }
        for (int j = 0; j < size; j++)
            c->act[l + 1][j] = is_real ? C(relu64(c->angle[l][j].re), 0.0) : lc64(c->angle[l][j]);
    }
    const int last = psi->size[psi->num_layers - 1];
    const double* fw = part == 2 ? psi->final_w_im : psi->final_w;
    cd r = C(0.0, 0.0);
    for (int j = 0; j < last; j++) {
        const cd f = is_real ? C(fw[j], 0.0) : cload(fw, j);
        r = cadd(r, cmul(c->act[psi->num_layers][j], f));
    }
    return r;
}

/* Spins_t<1>::rotate_left (include/Spins.h:280-285), single word only. */
static void rotate_left(const uint64_t* s, int shift, int N, uint64_t* out) {
    const uint64_t x = s[0];
    uint64_t y = shift == 0 ? x : ((x << shift) | (x >> (N - shift)));
    if (N < 64) y &= ((uint64_t)1 << N) - 1u;
    out[0] = y;
    for (int k = 1; k < OR_MAX_WORDS; k++) out[k] = 0;
}

static cd deep_log_psi(const or_psi* psi, int part, const uint64_t* s) {   /* PsiDeep.hpp:135-169 */
    deep_cache* c = (deep_cache*)malloc(sizeof(deep_cache));
    cd r = C(0.0, 0.0);
    if (psi->translational_invariance) {
        for (int shift = 0; shift < psi->N; shift++) {
            uint64_t sh[OR_MAX_WORDS];
            rotate_left(s, shift, psi->N, sh);
            r = cadd(r, deep_forward(psi, part, sh, c));
        }
        r = cscale(1.0 / psi->N, r);
    } else {
        r = deep_forward(psi, part, s, c);
    }
    free(c);
    return r;
}

void or_log_psi(const or_psi* psi, const uint64_t* spins, double* out) {
    cd r;
    if (psi->kind == OR_PSI_RBM) {                                          /* Psi.hpp:55-63 */
        r = C(0.0, 0.0);
        for (int j = 0; j < psi->M; j++) r = cadd(r, lc64(rbm_angle(psi, j, spins)));
    } else if (psi->kind == OR_PSI_DEEP) {
        r = deep_log_psi(psi, 0, spins);
    } else {                                                                /* PsiPair.hpp:47-51 */
        r = C(deep_log_psi(psi, 1, spins).re, deep_log_psi(psi, 2, spins).re);
    }
    out[0] = r.re;
    out[1] = r.im;
}

static cd log_psi_cd(const or_psi* psi, const uint64_t* s) {
    double o[2];
    or_log_psi(psi, s, o);
    return C(o[0], o[1]);
}

int or_num_params(const or_psi* psi) {
    if (psi->kind == OR_PSI_RBM) return 2 * psi->N + psi->M + psi->N * psi->M;   /* Psi.hpp:231-234 */
    int P = 2 * psi->N;                                                         /* PsiDeep.cu:34-66 */
    for (int l = 0; l < psi->num_layers; l++) P += psi->size[l] + psi->conn[l] * psi->size[l];
    return P + psi->size[psi->num_layers - 1];
}

/* Reverse pass of PsiDeep.hpp:214-293 (complex) or of the real nets of a PsiPair.
 * out receives [P] values (complex interleaved when complex_out). */
static void deep_O_k(const or_psi* psi, int part, const uint64_t* s, double* out, int complex_out) {
    const int is_real = psi->kind == OR_PSI_PAIR;
    deep_cache* c = (deep_cache*)malloc(sizeof(deep_cache));
    const cd log_psi = deep_forward(psi, part, s, c);
    const int L = psi->num_layers;
    const int P = or_num_params(psi);
    static cd back[2][DEEP_MAX_UNITS];
    int begin[OR_MAX_LAYERS];
    int k = 2 * psi->N;
    for (int l = 0; l < L; l++) { begin[l] = k; k += psi->size[l] + psi->conn[l] * psi->size[l]; }
    const double* fw = part == 2 ? psi->final_w_im : psi->final_w;
#define EMIT(idx, val) do { if (complex_out) cstore(out, (idx), (val)); else out[(idx)] = (val).re; } while (0)
    cd* cur = back[0];
    cd* nxt = back[1];
    for (int l = L - 1; l >= 0; l--) {
        const int size = psi->size[l];
        if (l == L - 1) {
            for (int j = 0; j < size; j++) {
                const cd f = is_real ? C(fw[j], 0.0) : cload(fw, j);
                const cd t = is_real ? C(1.0, 0.0) : tanh64(c->angle[l][j]);
                cur[j] = cmul(f, t);
            }
        } else {
            /* rhs sums in the order compile_rhs_connections_and_weights lists them
             * (source/quantum_state/PsiDeep.cu:101-111): next-layer unit j ascending */
            const int nsize = psi->size[l + 1], nconn = psi->conn[l + 1];
            const double *nw, *nb;
            deep_weights(psi, part, l + 1, &nw, &nb);
            for (int i = 0; i < size; i++) cur[i] = C(0.0, 0.0);
            for (int j = 0; j < nsize; j++)
                for (int ci = 0; ci < nconn; ci++) {
                    const unsigned src = psi->lhs_conn[l + 1][(long)ci * nsize + j];
                    const cd wij = is_real ? C(nw[(long)ci * nsize + j], 0.0) : cload(nw, (long)ci * nsize + j);
                    cur[src] = cadd(cur[src], cmul(wij, nxt[j]));
                }
            for (int i = 0; i < size; i++) {
                const cd t = is_real ? C(1.0, 0.0) : tanh64(c->angle[l][i]);
                cur[i] = cmul(cur[i], t);
            }
        }
        const int conn = psi->conn[l];
        for (int j = 0; j < size; j++) {
            EMIT(begin[l] + j, cur[j]);
            for (int i = 0; i < conn; i++) {
                const unsigned src = psi->lhs_conn[l][(long)i * size + j];
                const cd in = l == 0 ? C(spin_at(s, (int)src), 0.0) : c->act[l][src];
                EMIT(begin[l] + size + (long)i * size + j, cmul(cur[j], in));
            }
        }
        cd* tmp = cur; cur = nxt; nxt = tmp;
    }
    /* final weights: log_psi * activation of the last layer (PsiDeep.hpp:285-292) */
    const int last = psi->size[L - 1];
    for (int j = 0; j < last; j++) EMIT(P - last + j, cmul(log_psi, c->act[L][j]));
#undef EMIT
    free(c);
}

void or_O_k(const or_psi* psi, const uint64_t* spins, double* out) {
    const int P = or_num_params(psi);
    memset(out, 0, sizeof(double) * 2 * (size_t)P);
    if (psi->kind == OR_PSI_RBM) {                                   /* Psi.hpp:165-202 */
        const int N = psi->N, M = psi->M;
        for (int j = 0; j < M; j++) {
            const cd t = tanh64(rbm_angle(psi, j, spins));
            cstore(out, 2 * N + j, t);
            for (int i = 0; i < N; i++) cstore(out, 2 * N + M + (long)i * M + j, cscale(spin_at(spins, i), t));
        }
    } else if (psi->kind == OR_PSI_DEEP) {
        deep_O_k(psi, 0, spins, out, 1);
    }
    /* PsiPair::foreach_O_k is empty (PsiPair.hpp:73-76): zeros */
}

void or_O_k_pair(const or_psi* psi, int part, const uint64_t* spins, double* out) {
    memset(out, 0, sizeof(double) * (size_t)or_num_params(psi));
    deep_O_k(psi, part == 0 ? 1 : 2, spins, out, 0);
}

/* ------------------------------------------------------------------------- */
/* Operator (include/operator/Operator.hpp:45-179)                            */
/* ------------------------------------------------------------------------- */
/* nth_matrix_element: coefficient * phases (Y: -i s_i, Z: s_i with the ORIGINAL
 * spins) and the flipped configuration. */
static cd matrix_element(const or_op* op, int n, const uint64_t* s, uint64_t* s_prime, int nw) {
    cd coef = cload(op->coef, n);
    for (int k = 0; k < nw; k++) s_prime[k] = s[k];
    for (int col = 0; col < op->L; col++) {
        const int idx = op->idx[n * op->L + col];
        if (idx < 0) break;
        const int t = op->types[n * op->L + col];
        if (t == 1) {
            spin_flip(s_prime, idx);
        } else if (t == 2) {
            spin_flip(s_prime, idx);
            coef = cmul(coef, C(0.0, -spin_at(s, idx)));
        } else if (t == 3) {
            coef = cscale(spin_at(s, idx), coef);
        }
    }
    return coef;
}

void or_local_energy(const or_psi* psi, const or_op* op, const uint64_t* spins, const double* log_psi, double* out) {
    const int nw = nwords_of(psi->N);
    const cd lp = C(log_psi[0], log_psi[1]);
    cd e = C(0.0, 0.0);
    for (int n = 0; n < op->S; n++) {                               /* Operator.hpp:90-115 */
        uint64_t sp[OR_MAX_WORDS] = {0};
        const cd coef = matrix_element(op, n, spins, sp, nw);
        if (spins_equal(sp, spins, nw)) {
            e = cadd(e, coef);
        } else {
            e = cadd(e, cmul(coef, cexp_(csub(log_psi_cd(psi, sp), lp))));
        }
    }
    out[0] = e.re;
    out[1] = e.im;
}

void or_E_k_accumulate(const or_psi* psi, const or_op* op, const uint64_t* spins, const double* log_psi,
                       double weight, double* acc) {
    const int nw = nwords_of(psi->N);
    const int P = or_num_params(psi);
    const cd lp = C(log_psi[0], log_psi[1]);
    double* ok = (double*)malloc(sizeof(double) * 2 * (size_t)P);
    for (int n = 0; n < op->S; n++) {                               /* Operator.hpp:145-179 */
        uint64_t sp[OR_MAX_WORDS] = {0};
        const cd coef = matrix_element(op, n, spins, sp, nw);
        cd e = coef;
        if (!spins_equal(sp, spins, nw)) e = cmul(coef, cexp_(csub(log_psi_cd(psi, sp), lp)));
        or_O_k(psi, sp, ok);
        const cd we = cscale(weight, e);
        for (int k = 0; k < P; k++) cacc(acc, k, cmul(we, cload(ok, k)));
    }
    free(ok);
}

/* ------------------------------------------------------------------------- */
/* exact summation (include/spin_ensembles/ExactSummation.hpp:36-84)          */
/* ------------------------------------------------------------------------- */
static inline void index_spins(uint64_t idx, int N, uint64_t* s) {   /* Spins_t<1>(idx, N) */
    for (int k = 0; k < OR_MAX_WORDS; k++) s[k] = 0;
    s[0] = N >= 64 ? idx : (idx & (((uint64_t)1 << N) - 1u));
}

static inline double ref_weight(const or_psi* psi, cd lp) {          /* probability_s, include/quantum_state/Psi.hpp:134-137 */
    return exp(2.0 * (log(psi->prefactor) + lp.re));
}

double or_exact_norm(const or_psi* psi) {                            /* PsiNorm.cu:13-44 */
    double sum = 0.0;
    const uint64_t dim = (uint64_t)1 << psi->N;
    for (uint64_t x = 0; x < dim; x++) {
        uint64_t s[OR_MAX_WORDS];
        index_spins(x, psi->N, s);
        sum += ref_weight(psi, log_psi_cd(psi, s));
    }
    return sqrt(sum);
}

void or_psi_vector(const or_psi* psi, double* out) {                 /* PsiVector.cu:13-51 */
    const uint64_t dim = (uint64_t)1 << psi->N;
    const double lpf = log(psi->prefactor);
    for (uint64_t x = 0; x < dim; x++) {
        uint64_t s[OR_MAX_WORDS];
        index_spins(x, psi->N, s);
        cd lp = log_psi_cd(psi, s);
        lp.re += lpf;
        cstore(out, (long)x, cexp_(lp));
    }
}

void or_exact_fluctuation(const or_psi* psi, const or_op* op, double* E, double* sigma) {
    const uint64_t dim = (uint64_t)1 << psi->N;
    cd e = C(0.0, 0.0);
    double e2 = 0.0;
    for (uint64_t x = 0; x < dim; x++) {
        uint64_t s[OR_MAX_WORDS];
        index_spins(x, psi->N, s);
        const cd lp = log_psi_cd(psi, s);
        const double w = ref_weight(psi, lp);
        double el[2];
        const double lpa[2] = {lp.re, lp.im};
        or_local_energy(psi, op, s, lpa, el);
        e = cadd(e, cscale(w, C(el[0], el[1])));
        e2 += w * (el[0] * el[0] + el[1] * el[1]);
    }
    E[0] = e.re;
    E[1] = e.im;
    if (sigma) *sigma = sqrt(e2 - cnorm(e));                         /* ExpectationValue.cu:171-174 */
}

void or_exact_value(const or_psi* psi, const or_op* op, double* E) { or_exact_fluctuation(psi, op, E, NULL); }

/* Accumulators of ExpectationValue::gradient (ExpectationValue.cu:177-256). */
typedef struct { int P; cd E; double* O; double* EO; double* Ek; double wsum; } grad_acc;

static void grad_acc_init(grad_acc* a, int P) {
    a->P = P;
    a->E = C(0.0, 0.0);
    a->O = (double*)calloc(2 * (size_t)P, sizeof(double));
    a->EO = (double*)calloc(2 * (size_t)P, sizeof(double));
    a->Ek = (double*)calloc(2 * (size_t)P, sizeof(double));
}

static void grad_acc_add(grad_acc* a, const or_psi* psi, const or_op* op, const uint64_t* s, cd lp, double w, double* ok) {
    double el[2];
    const double lpa[2] = {lp.re, lp.im};
    or_local_energy(psi, op, s, lpa, el);
    const cd e = C(el[0], el[1]);
    a->E = cadd(a->E, cscale(w, e));
    or_O_k(psi, s, ok);
    for (int k = 0; k < a->P; k++) {
        const cd o = cload(ok, k);
        cacc(a->O, k, cscale(w, o));
        cacc(a->EO, k, cmul(cscale(w, e), cconj(o)));
    }
    or_E_k_accumulate(psi, op, s, lpa, w, a->Ek);
}

static void grad_acc_finish(grad_acc* a, double inv_steps, double* grad, double* E) {
    const cd Eavg = cscale(inv_steps, a->E);
    for (int k = 0; k < a->P; k++) {
        const cd o = cscale(inv_steps, cload(a->O, k));
        const cd eo = cscale(inv_steps, cload(a->EO, k));
        const cd ek = cscale(inv_steps, cload(a->Ek, k));
        cstore(grad, k, csub(cadd(eo, cconj(ek)), cscale(2.0, cmul(Eavg, cconj(o)))));
    }
    E[0] = Eavg.re;
    E[1] = Eavg.im;
    free(a->O); free(a->EO); free(a->Ek);
}

void or_exact_gradient(const or_psi* psi, const or_op* op, double* grad, double* E) {
    const int P = or_num_params(psi);
    const uint64_t dim = (uint64_t)1 << psi->N;
    double* ok = (double*)malloc(sizeof(double) * 2 * (size_t)P);
    grad_acc a;
    grad_acc_init(&a, P);
    for (uint64_t x = 0; x < dim; x++) {
        uint64_t s[OR_MAX_WORDS];
        index_spins(x, psi->N, s);
        const cd lp = log_psi_cd(psi, s);
        grad_acc_add(&a, psi, op, s, lp, ref_weight(psi, lp), ok);
    }
    free(ok);
    grad_acc_finish(&a, 1.0, grad, E);
}

void or_samples_gradient(const or_psi* psi, const or_op* op, int num_samples, const uint64_t* spins,
                         double* grad, double* E) {
    const int P = or_num_params(psi);
    const int nw = nwords_of(psi->N);
    double* ok = (double*)malloc(sizeof(double) * 2 * (size_t)P);
    grad_acc a;
    grad_acc_init(&a, P);
    for (int t = 0; t < num_samples; t++) {
        const uint64_t* s = spins + (size_t)t * nw;
        grad_acc_add(&a, psi, op, s, log_psi_cd(psi, s), 1.0, ok);
    }
    free(ok);
    grad_acc_finish(&a, 1.0 / num_samples, grad, E);
}

/* ------------------------------------------------------------------------- */
/* Hilbert-space distance (source/network_functions/HilbertSpaceDistance.cu:14-269,
 * PsiPair gradient HilbertSpaceDistance_PsiPair.cu:14-173)                   */
/* ------------------------------------------------------------------------- */
typedef struct { cd omega; double pr; double nn; double* omega_O; double* pr_O; } hsd_acc;

static inline double qa_at(const double* a, int i) { return a ? a[i] : 0.0; }

/* part: -1 general complex O_k of psi_prime; 0/1 PsiPair real/imag net O_k (real).
 * With psi's free quantum axis (HilbertSpaceDistance.cu:47-81, 109-122; part -1 only, the
 * PsiPair gradient of HilbertSpaceDistance_PsiPair.cu has no such branch): r_i =
 * psi'(s with spin i flipped) / psi'(s), log psi'(s) += sum_i [da_i s_i r_i +
 * i db_i (r_i cos(sa_i) - s_i sin(sa_i))] with da = alpha' - alpha, db = beta' - beta,
 * sa = alpha' + alpha, and the O_k of alpha_i, beta_i are s_i r_i, i (r_i cos - s_i sin). */
static void hsd_add(hsd_acc* h, const or_psi* psi, const or_psi* pp, const or_op* op, int is_unitary,
                    const uint64_t* s, double w, int want_grad, int part, double* ok) {
    const cd lp = log_psi_cd(psi, s);
    double el[2];
    const double lpa[2] = {lp.re, lp.im};
    or_local_energy(psi, op, s, lpa, el);
    const cd e = C(el[0], el[1]);
    cd lpp = log_psi_cd(pp, s);
    const int fqa = psi->free_quantum_axis && part < 0;
    const int N = psi->N;
    cd* qa_o = NULL;   /* [2N] the alpha / beta O_k of this sample */
    if (fqa) {
        qa_o = (cd*)malloc(sizeof(cd) * 2 * (size_t)N);
        cd corr = C(0.0, 0.0);
        for (int i = 0; i < N; i++) {
            uint64_t si[OR_MAX_WORDS];
            memcpy(si, s, sizeof(uint64_t) * nwords_of(N));
            spin_flip(si, i);
            const cd r = cexp_(csub(log_psi_cd(pp, si), lpp));
            const double sg = spin_at(s, i);
            const double da = qa_at(pp->alpha, i) - qa_at(psi->alpha, i);
            const double db = qa_at(pp->beta, i) - qa_at(psi->beta, i);
            const double sa = qa_at(pp->alpha, i) + qa_at(psi->alpha, i);
            const cd oa = cscale(sg, r);
            const cd ob = cmul(C(0.0, 1.0), csub(cscale(cos(sa), r), C(sg * sin(sa), 0.0)));
            qa_o[i] = oa;
            qa_o[N + i] = ob;
            corr = cadd(corr, cadd(cscale(da, oa), cscale(db, ob)));
        }
        lpp = cadd(lpp, corr);
    }
    cd omega;
    if (is_unitary) {
        omega = cmul(cexp_(cconj(csub(lpp, lp))), e);
        h->nn += w * cnorm(e);
    } else {
        omega = cexp_(cadd(e, cconj(csub(lpp, lp))));
        h->nn += w * exp(2.0 * e.re);
    }
    const double pr = exp(2.0 * (lpp.re - lp.re));
    h->omega = cadd(h->omega, cscale(w, omega));
    h->pr += w * pr;
    if (!want_grad) { free(qa_o); return; }
    const int P = or_num_params(pp);
    if (part < 0) {
        or_O_k(pp, s, ok);
        if (fqa)
            for (int k = 0; k < 2 * N; k++) cstore(ok, k, qa_o[k]);
        free(qa_o);
        for (int k = 0; k < P; k++) {
            const cd oc = cconj(cload(ok, k));
            cacc(h->omega_O, k, cmul(cscale(w, omega), oc));
            cacc(h->pr_O, k, cscale(w * pr, oc));
        }
    } else {
        or_O_k_pair(pp, part, s, ok);
        for (int k = 0; k < P; k++) {
            cacc(h->omega_O, k, cscale(w * ok[k], omega));
            if (part == 0) cacc(h->pr_O, k, C(w * pr * ok[k], 0.0));
        }
    }
}

typedef struct {
    const or_psi* psi;
    int exact;          /* 1: all 2^N states with reference weights; 0: equal weights over samples */
    int num_samples;
    const uint64_t* spins;
} ensemble;

static void hsd_run(hsd_acc* h, const ensemble* ens, const or_psi* pp, const or_op* op, int is_unitary,
                    int want_grad, int part) {
    const or_psi* psi = ens->psi;
    const int P = or_num_params(pp);
    memset(h, 0, sizeof(*h));
    h->omega_O = (double*)calloc(2 * (size_t)P, sizeof(double));
    h->pr_O = (double*)calloc(2 * (size_t)P, sizeof(double));
    double* ok = (double*)malloc(sizeof(double) * 2 * (size_t)P);
    if (ens->exact) {
        const uint64_t dim = (uint64_t)1 << psi->N;
        for (uint64_t x = 0; x < dim; x++) {
            uint64_t s[OR_MAX_WORDS];
            index_spins(x, psi->N, s);
            hsd_add(h, psi, pp, op, is_unitary, s, ref_weight(psi, log_psi_cd(psi, s)), want_grad, part, ok);
        }
    } else {
        const int nw = nwords_of(psi->N);
        for (int t = 0; t < ens->num_samples; t++)
            hsd_add(h, psi, pp, op, is_unitary, ens->spins + (size_t)t * nw, 1.0, want_grad, part, ok);
        const double inv = 1.0 / ens->num_samples;
        h->omega = cscale(inv, h->omega);
        h->pr *= inv;
        h->nn *= inv;
        for (int k = 0; k < 2 * P; k++) { h->omega_O[k] *= inv; h->pr_O[k] *= inv; }
    }
    free(ok);
}

static double hsd_distance_and_gradient(const ensemble* ens, const or_psi* pp, const or_op* op, int is_unitary,
                                        double nu, double* grad) {
    const int P = or_num_params(pp);
    hsd_acc h;
    if (pp->kind == OR_PSI_PAIR && grad) {
        /* two passes: real net then imaginary net (HilbertSpaceDistance_PsiPair.cu:99-169) */
        hsd_run(&h, ens, pp, op, is_unitary, 1, 0);
        double u = cnorm(h.omega), v = h.nn * h.pr;
        double dist = sqrt(1.0 - u / v);
        for (int k = 0; k < P; k++) {
            const double uk = 2.0 * cmul(cconj(h.omega), cload(h.omega_O, k)).re;
            const double vk = 2.0 * (h.nn * h.pr_O[2 * k]);
            cstore(grad, k, C((-0.5 * (uk * v - u * vk) / (v * v)) / dist, 0.0));
        }
        free(h.omega_O); free(h.pr_O);
        hsd_run(&h, ens, pp, op, is_unitary, 1, 1);
        u = cnorm(h.omega); v = h.nn * h.pr;
        dist = sqrt(1.0 - u / v);
        for (int k = 0; k < P; k++) {
            const double uk = 2.0 * cmul(cconj(h.omega), cload(h.omega_O, k)).im;
            grad[2 * k + 1] += (-0.5 * uk / v) / dist;
        }
        free(h.omega_O); free(h.pr_O);
        return dist;
    }
    hsd_run(&h, ens, pp, op, is_unitary, grad != NULL, -1);
    const double u = cnorm(h.omega);
    const double v = h.nn * h.pr;
    const double dist = sqrt(1.0 - u / v);
    if (grad) {
        const double pf = pow(dist, nu);
        for (int k = 0; k < P; k++) {
            const cd uk = cmul(cconj(h.omega), cload(h.omega_O, k));
            const cd vk = cscale(h.nn, cload(h.pr_O, k));
            const cd g = cscale(-1.0 / (v * v), csub(cscale(v, uk), cscale(u, vk)));
            cstore(grad, k, cscale(1.0 / pf, g));
        }
    }
    free(h.omega_O); free(h.pr_O);
    return dist;
}

double or_exact_hsd(const or_psi* psi, const or_psi* psi_prime, const or_op* op, int is_unitary,
                    double nu, double* grad) {
    ensemble e = {psi, 1, 0, NULL};
    return hsd_distance_and_gradient(&e, psi_prime, op, is_unitary, nu, grad);
}

double or_samples_hsd(const or_psi* psi, const or_psi* psi_prime, const or_op* op, int is_unitary,
                      int num_samples, const uint64_t* spins, double nu, double* grad) {
    ensemble e = {psi, 0, num_samples, spins};
    return hsd_distance_and_gradient(&e, psi_prime, op, is_unitary, nu, grad);
}

/* ------------------------------------------------------------------------- */
/* Metropolis (include/spin_ensembles/MonteCarloLoop.hpp:55-256)              */
/* ------------------------------------------------------------------------- */
typedef struct {
    const or_psi* psi;
    const or_mc_cfg* cfg;
    rng_t rng;
    int nw;
    uint64_t s[OR_MAX_WORDS];
    /* FP64 reference mode */
    cd* theta;
    double log_psi_real;
    /* FP32 GPU-spec mode */
    float* th_r;
    float* th_i;
    float* re;
    float* tr_r;
    float* tr_i;
    float* tre;
    uint64_t acc, rej;
} chain_t;

static double ref_log_psi_real(chain_t* c) {                      /* Psi.hpp:229-250 (host) */
    const or_psi* psi = c->psi;
    if (psi->kind == OR_PSI_RBM) {
        double r = 0.0;
        for (int j = 0; j < psi->M; j++) r += lc64(c->theta[j]).re;
        return r;
    }
    return log_psi_cd(psi, c->s).re;          /* PsiDeep / PsiPair: forward pass from the spins */
}

static void ref_flip_angles(chain_t* c, int pos) {                 /* Psi.hpp:252-258 */
    const or_psi* psi = c->psi;
    if (psi->kind != OR_PSI_RBM) return;
    const double sv = spin_at(c->s, pos);
    for (int j = 0; j < psi->M; j++)
        c->theta[j] = cadd(c->theta[j], cscale(2.0 * sv, cload(psi->W, (long)pos * psi->M + j)));
}

static void ref_mc_update(chain_t* c) {                            /* MonteCarloLoop.hpp:153-256 */
    const or_psi* psi = c->psi;
    const or_mc_cfg* cfg = c->cfg;
    const int N = psi->N;
    uint64_t original[OR_MAX_WORDS];
    int position = 0, second = 0;
    if (cfg->fast_sweep_tries > 0) {
        memcpy(original, c->s, sizeof(original));
        uint64_t mask[OR_MAX_WORDS] = {0}, m2[OR_MAX_WORDS] = {0};
        rng_spins(&c->rng, N, mask);
        for (int t = 1; t < cfg->fast_sweep_tries; t++) {
            rng_spins(&c->rng, N, m2);
            for (int k = 0; k < c->nw; k++) mask[k] &= m2[k];
        }
        for (int k = 0; k < c->nw; k++) c->s[k] ^= mask[k];
        /* the reference updates no angles here (its Psi keeps stale angles) */
    } else {
        position = (int)(rng_u32(&c->rng) % (uint32_t)N);
        spin_flip(c->s, position);
        ref_flip_angles(c, position);
    }
    if (cfg->total_z) {
        for (;;) {
            second = (int)(rng_u32(&c->rng) % (uint32_t)N);
            if (spin_at(c->s, second) == spin_at(c->s, position)) { spin_flip(c->s, second); break; }
        }
        ref_flip_angles(c, second);
    }
    const double next = ref_log_psi_real(c);
    const double ratio = exp(2.0 * (next - c->log_psi_real));
    if (ratio > 1.0 || rng_real(&c->rng) <= ratio) {
        c->log_psi_real = next;
        c->acc++;
    } else {
        c->rej++;
        if (cfg->fast_sweep_tries > 0) {
            memcpy(c->s, original, sizeof(original));
        } else {
            spin_flip(c->s, position);
            ref_flip_angles(c, position);
        }
        if (cfg->total_z) {
            spin_flip(c->s, second);
            ref_flip_angles(c, second);
        }
    }
}

/* ---- FP32 GPU-spec chain (rbmongpu_gb300/csrc/mc_rbm.cu) ---- */
static inline int mpad32(int M) { return (M + 31) / 32 * 32; }

/* angles from scratch: theta_j = b_j, then theta_j +/-= W_ij for i = 0..N-1 */
static void g32_refresh(chain_t* c) {
    const or_psi* psi = c->psi;
    const int M = psi->M;
    for (int j = 0; j < M; j++) {
        float tr = (float)psi->b[2 * j], ti = (float)psi->b[2 * j + 1];
        for (int i = 0; i < psi->N; i++) {
            const float wr = (float)psi->W[2 * ((long)i * M + j)];
            const float wi = (float)psi->W[2 * ((long)i * M + j) + 1];
            if (spin_at(c->s, i) > 0) { tr = tr + wr; ti = ti + wi; }
            else { tr = tr - wr; ti = ti - wi; }
        }
        c->th_r[j] = tr;
        c->th_i[j] = ti;
        c->re[j] = or_lc_re_f32(tr, ti);
    }
}

/* per-lane partial sums over j = lane + 32 k, then the xor butterfly 16,8,4,2,1 */
static float warp_sum32(const float* v, int M) {
    float part[32];
    for (int l = 0; l < 32; l++) {
        float a = 0.0f;
        for (int j = l; j < M; j += 32) a = a + v[j];
        part[l] = a;
    }
    for (int off = 16; off >= 1; off >>= 1) {
        float nx[32];
        for (int l = 0; l < 32; l++) nx[l] = part[l] + part[l ^ off];
        memcpy(part, nx, sizeof(part));
    }
    return part[0];
}

static int g32_try(chain_t* c, const int* sites, int nsites) {
    const or_psi* psi = c->psi;
    const int M = psi->M;
    uint64_t s2[OR_MAX_WORDS];
    memcpy(s2, c->s, sizeof(s2));
    for (int j = 0; j < M; j++) { c->tr_r[j] = c->th_r[j]; c->tr_i[j] = c->th_i[j]; }
    for (int q = 0; q < nsites; q++) {
        const int pos = sites[q];
        spin_flip(s2, pos);
        const float two_s = spin_at(s2, pos) > 0 ? 2.0f : -2.0f;
        for (int j = 0; j < M; j++) {
            c->tr_r[j] = fmaf(two_s, (float)psi->W[2 * ((long)pos * M + j)], c->tr_r[j]);
            c->tr_i[j] = fmaf(two_s, (float)psi->W[2 * ((long)pos * M + j) + 1], c->tr_i[j]);
        }
    }
    float* d = c->tre + M;   /* scratch after tre[0..M) */
    for (int j = 0; j < M; j++) {
        c->tre[j] = or_lc_re_f32(c->tr_r[j], c->tr_i[j]);
        d[j] = c->tre[j] - c->re[j];
    }
    const float delta = warp_sum32(d, M);
    int accept = delta > 0.0f;
    if (!accept) {
        const float u = (float)rng_real(&c->rng);
        accept = u <= or_expf_det(2.0f * delta);
    }
    if (accept) {
        memcpy(c->s, s2, sizeof(s2));
        for (int j = 0; j < M; j++) { c->th_r[j] = c->tr_r[j]; c->th_i[j] = c->tr_i[j]; c->re[j] = c->tre[j]; }
        c->acc++;
    } else {
        c->rej++;
    }
    return accept;
}

static void g32_mc_update(chain_t* c) {
    const int N = c->psi->N;
    int sites[2];
    int ns = 1;
    sites[0] = (int)(rng_u32(&c->rng) % (uint32_t)N);
    if (c->cfg->total_z) {
        const double first_new = -spin_at(c->s, sites[0]);
        for (;;) {
            const int sec = (int)(rng_u32(&c->rng) % (uint32_t)N);
            const double v = sec == sites[0] ? first_new : spin_at(c->s, sec);
            if (v == first_new) { sites[1] = sec; ns = 2; break; }
        }
    }
    g32_try(c, sites, ns);
}

/* fast sweep of the GPU spec (rbm_impl.cuh::rbm_fast_step2): the mask is the AND of
 * fast_sweep_tries random configurations; its sites in increasing order form one proposal */
static void g32_fast_update(chain_t* c) {
    const int N = c->psi->N;
    uint64_t mask[OR_MAX_WORDS] = {0}, m2[OR_MAX_WORDS] = {0};
    int sites[OR_MAX_WORDS * 64];
    int ns = 0;
    rng_spins(&c->rng, N, mask);
    for (int t = 1; t < c->cfg->fast_sweep_tries; t++) {
        rng_spins(&c->rng, N, m2);
        for (int k = 0; k < c->nw; k++) mask[k] &= m2[k];
    }
    for (int k = 0; k < c->nw; k++)
        for (int b = 0; b < 64; b++)
            if ((mask[k] >> b) & 1u) sites[ns++] = 64 * k + b;
    g32_try(c, sites, ns);
}

static void chain_init_spins(chain_t* c) {
    const or_psi* psi = c->psi;
    memset(c->s, 0, sizeof(c->s));
    if (c->cfg->total_z) {                                        /* MonteCarloLoop.hpp:79-90 */
        c->s[0] = rng_n_over_k(&c->rng, (unsigned)psi->N, (unsigned)((c->cfg->sector + psi->N) / 2));
        if (psi->N < 64) c->s[0] &= ((uint64_t)1 << psi->N) - 1u;
    } else {
        rng_spins(&c->rng, psi->N, c->s);
    }
}

int or_mc_run(const or_psi* psi, const or_op* op, const or_mc_cfg* cfg,
              uint64_t* spins_out, double* log_psi_out, double* eloc_out,
              uint64_t* accepts, uint64_t* rejects) {
    if (cfg->prec == OR_PREC_GPU32 && psi->kind != OR_PSI_RBM) return -1;
    if (cfg->prec == OR_PREC_GPU32 && cfg->fast_sweep_tries > 0 && cfg->total_z) return -1;
    const int N = psi->N;
    const int nw = nwords_of(N);
    const int M = psi->kind == OR_PSI_RBM ? psi->M : 0;
    for (int cc = 0; cc < cfg->num_chains; cc++) {
        const int chain = cfg->chain_begin + cc;
        chain_t c;
        memset(&c, 0, sizeof(c));
        c.psi = psi;
        c.cfg = cfg;
        c.nw = nw;
        c.rng.kind = cfg->rng;
        if (cfg->rng == OR_RNG_MT19937) mt_seed(&c.rng.mt, (uint32_t)chain);
        c.rng.seed = cfg->seed;
        c.rng.walker = (uint32_t)chain;
        c.rng.index = 0;
        if (M > 0) {
            c.theta = (cd*)malloc(sizeof(cd) * (size_t)M);
            c.th_r = (float*)malloc(sizeof(float) * (size_t)mpad32(M) * 7);
            c.th_i = c.th_r + mpad32(M);
            c.re = c.th_i + mpad32(M);
            c.tr_r = c.re + mpad32(M);
            c.tr_i = c.tr_r + mpad32(M);
            c.tre = c.tr_i + mpad32(M);
        }
        if (cfg->state_spins && cfg->resume) {
            memcpy(c.s, cfg->state_spins + (size_t)cc * nw, sizeof(uint64_t) * nw);
            c.rng.index = cfg->state_rng[cc];
        } else {
            chain_init_spins(&c);
        }
        const int fast = cfg->fast_sweep_tries > 0;
        if (cfg->prec == OR_PREC_REF64) {
            if (M > 0) for (int j = 0; j < M; j++) c.theta[j] = rbm_angle(psi, j, c.s);
            c.log_psi_real = ref_log_psi_real(&c);
            for (long t = 0; t < (long)cfg->num_therm * N; t++) ref_mc_update(&c);
        } else {
            for (int t = 0; t < cfg->num_therm; t++) {
                g32_refresh(&c);
                for (int p = 0; p < N; p++) {
                    if (fast) g32_fast_update(&c);
                    else g32_mc_update(&c);
                }
            }
        }
        for (int step = 0; step < cfg->samples_per_chain; step++) {
            if (cfg->prec == OR_PREC_REF64) {
                const long nupd = (long)cfg->num_sweeps * (fast ? 1 : N);
                for (long t = 0; t < nupd; t++) ref_mc_update(&c);
            } else if (fast) {
                /* one update per sweep; angles from scratch at the sample's start and every N updates */
                for (int t = 0; t < cfg->num_sweeps; t++) {
                    if (t % N == 0) g32_refresh(&c);
                    g32_fast_update(&c);
                }
            } else {
                for (int t = 0; t < cfg->num_sweeps; t++) {
                    g32_refresh(&c);
                    for (int p = 0; p < N; p++) g32_mc_update(&c);
                }
            }
            const size_t o = (size_t)step * cfg->num_chains + cc;
            if (spins_out) memcpy(spins_out + o * nw, c.s, sizeof(uint64_t) * nw);
            double lp[2];
            if (log_psi_out || (eloc_out && op)) {
                if (psi->kind == OR_PSI_RBM && cfg->prec == OR_PREC_REF64) {
                    cd r = C(0.0, 0.0);                    /* log psi from the chain's angles */
                    for (int j = 0; j < M; j++) r = cadd(r, lc64(c.theta[j]));
                    lp[0] = r.re; lp[1] = r.im;
                } else {
                    or_log_psi(psi, c.s, lp);
                }
            }
            if (log_psi_out) { log_psi_out[2 * o] = lp[0]; log_psi_out[2 * o + 1] = lp[1]; }
            if (eloc_out && op) or_local_energy(psi, op, c.s, lp, eloc_out + 2 * o);
        }
        if (accepts) accepts[cc] = c.acc;
        if (rejects) rejects[cc] = c.rej;
        if (cfg->state_spins) {
            memcpy(cfg->state_spins + (size_t)cc * nw, c.s, sizeof(uint64_t) * nw);
            cfg->state_rng[cc] = c.rng.index;
        }
        free(c.theta);
        free(c.th_r);
    }
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Learned-proposal chain, FP32 replay of rbmongpu_gb300/csrc/proposal.cu    */
/* (learned_draw_kernel, learned_accept_kernel): the step of                 */
/* include/spin_ensembles/MonteCarloLoop.hpp:206-222 with a cluster proposal */
/* and the Metropolis-Hastings density ratio.  The proposal has no reference */
/* counterpart; this replays the device's operation order so that a test    */
/* fed the device's logits checks every draw and decision bit for bit.       */
/* ------------------------------------------------------------------------- */
#define LR_LENGTHS 8

/* the xor butterfly 16, 8, 4, 2, 1 of device_math.cuh::warp_sum_xor */
static float butterfly32(float* part) {
    for (int off = 16; off >= 1; off >>= 1) {
        float nx[32];
        for (int l = 0; l < 32; l++) nx[l] = part[l] + part[l ^ off];
        memcpy(part, nx, sizeof(nx));
    }
    return part[0];
}

typedef struct { float seed, len; } lr_norm;

/* proposal.cu::log_norms_of: lane l sums the seed terms j = l + 32 c in c order */
static lr_norm lr_log_norms(const float* row, int N) {
    float m = -INFINITY, m2 = -INFINITY;
    for (int j = 0; j < N; j++) m = fmaxf(m, row[j]);
    for (int q = 0; q < LR_LENGTHS; q++) m2 = fmaxf(m2, row[N + q]);
    float part[32], part2[32];
    for (int l = 0; l < 32; l++) {
        float a = 0.0f;
        for (int c = 0; c < 8; c++)
            if (l + 32 * c < N) a = a + or_expf_det(row[l + 32 * c] - m);
        part[l] = a;
        part2[l] = l < LR_LENGTHS ? or_expf_det(row[N + l] - m2) : 0.0f;
    }
    lr_norm r;
    r.seed = m + or_logf_det(butterfly32(part));
    r.len = m2 + or_logf_det(butterfly32(part2));
    return r;
}

/* proposal.cu::draw_index: inverse CDF in chunks of 32, Hillis-Steele inclusive scan */
static int lr_draw(const float* row, int n, float lse, float u) {
    float base = 0.0f;
    int last = 0;
    for (int c = 0; c < n; c += 32) {
        float e[32], x[32], y[32];
        for (int l = 0; l < 32; l++) {
            e[l] = c + l < n ? or_expf_det(row[c + l] - lse) : 0.0f;
            x[l] = e[l];
        }
        for (int off = 1; off < 32; off <<= 1) {
            memcpy(y, x, sizeof(y));
            for (int l = off; l < 32; l++) x[l] = x[l] + y[l - off];
        }
        for (int l = 0; l < 32; l++)
            if (e[l] > 0.0f && base + x[l] >= u) return c + l;
        for (int l = 31; l >= 0; l--)
            if (e[l] > 0.0f) { last = c + l; break; }
        base = base + x[31];
    }
    return last;
}

static inline float lr_log_q(const float* row, int N, int i, int l, lr_norm ln) {
    return (row[i] - ln.seed) + (row[N + l - 1] - ln.len);
}

static inline float lr_uniform(rng_t* r) { return (float)rng_real(r); }

int or_learned_replay(int N, int M, int Mpad, const float* Wr, const float* Wi, int B, int steps, uint64_t seed,
                      uint32_t walker_base, const uint64_t* spins0, const uint64_t* rng0, const float* theta0,
                      const float* re0, const float* logits0, const float* logits_prop, int* site, int* len,
                      float* logq, uint64_t* spins_out, uint8_t* accepted, uint64_t* rng_end) {
    const int nw = nwords_of(N), O = N + LR_LENGTHS, K = Mpad / 32;
    if (N <= LR_LENGTHS || nw > OR_MAX_WORDS || Mpad % 32 || M > Mpad) return -1;
    float* tr = (float*)malloc(sizeof(float) * 6 * Mpad);
    float* cur = (float*)malloc(sizeof(float) * O);
    if (!tr || !cur) { free(tr); free(cur); return -2; }
    float *ti = tr + Mpad, *re = tr + 2 * Mpad, *nr = tr + 3 * Mpad, *ni = tr + 4 * Mpad, *nre = tr + 5 * Mpad;
    for (int w = 0; w < B; w++) {
        uint64_t s[OR_MAX_WORDS] = {0};
        memcpy(s, spins0 + (size_t)w * nw, sizeof(uint64_t) * nw);
        rng_t rng;
        memset(&rng, 0, sizeof(rng));
        rng.kind = OR_RNG_PHILOX;
        rng.seed = seed;
        rng.walker = walker_base + (uint32_t)w;
        rng.index = rng0[w];
        for (int j = 0; j < Mpad; j++) {
            tr[j] = theta0[((size_t)w * Mpad + j) * 2];
            ti[j] = theta0[((size_t)w * Mpad + j) * 2 + 1];
            re[j] = re0[(size_t)w * Mpad + j];
        }
        memcpy(cur, logits0 + (size_t)w * O, sizeof(float) * O);
        /* the first move, drawn from the current state's logits */
        lr_norm ln = lr_log_norms(cur, N);
        int i = lr_draw(cur, N, ln.seed, lr_uniform(&rng));
        int l = 1 + lr_draw(cur + N, LR_LENGTHS, ln.len, lr_uniform(&rng));
        float lq = lr_log_q(cur, N, i, l, ln);
        for (int t = 0; t < steps; t++) {
            const size_t o = (size_t)t * B + w;
            site[o] = i;
            len[o] = l;
            logq[o] = lq;
            const float* prop = logits_prop + o * O;
            /* trial angles: 2 s'_c W_c added in cluster order (s' = the flipped spin) */
            for (int j = 0; j < Mpad; j++) { nr[j] = tr[j]; ni[j] = ti[j]; }
            for (int q = 0; q < l; q++) {
                const int c = (i + q) % N;
                const float ts = spin_at(s, c) > 0 ? -2.0f : 2.0f;
                for (int j = 0; j < Mpad; j++) {       /* rows zero-padded to Mpad, as on the device */
                    nr[j] = fmaf(ts, j < M ? Wr[(size_t)c * M + j] : 0.0f, nr[j]);
                    ni[j] = fmaf(ts, j < M ? Wi[(size_t)c * M + j] : 0.0f, ni[j]);
                }
            }
            float part[32];
            for (int ln_ = 0; ln_ < 32; ln_++) {
                float a = 0.0f;
                for (int k = 0; k < K; k++) {
                    const int j = ln_ + 32 * k;
                    nre[j] = or_lc_re_f32(nr[j], ni[j]);
                    a = a + (nre[j] - re[j]);
                }
                part[ln_] = a;
            }
            const float delta = butterfly32(part);
            const lr_norm lp = lr_log_norms(prop, N);
            const float lq_rev = lr_log_q(prop, N, i, l, lp);
            const float log_a = fmaf(2.0f, delta, lq_rev) - lq;
            const float a = log_a >= 0.0f ? 1.0f : or_expf_det(log_a);
            int acc = log_a >= 0.0f;
            if (!acc) acc = lr_uniform(&rng) <= a;
            if (acc) {
                for (int j = 0; j < Mpad; j++) { tr[j] = nr[j]; ti[j] = ni[j]; re[j] = nre[j]; }
                memcpy(cur, prop, sizeof(float) * O);
                for (int q = 0; q < l; q++) spin_flip(s, (i + q) % N);
            }
            accepted[o] = (uint8_t)acc;
            memcpy(spins_out + o * nw, s, sizeof(uint64_t) * nw);
            if (t + 1 < steps) {
                ln = acc ? lp : lr_log_norms(cur, N);
                i = lr_draw(cur, N, ln.seed, lr_uniform(&rng));
                l = 1 + lr_draw(cur + N, LR_LENGTHS, ln.len, lr_uniform(&rng));
                lq = lr_log_q(cur, N, i, l, ln);
            }
        }
        rng_end[w] = rng.index;
    }
    free(tr);
    free(cur);
    return 0;
}
