// Elements of the per-sample O_k rows of an S-matrix chunk (SmSource), shared by the FP32
// tile kernel (smatrix.cu) and the tensor-core operand pass (smatrix_tc.cu).
#pragma once

#include "smatrix.h"

namespace rbmg {

struct SmElem {
    int i, j;   // RBM: spin index (-1: bias block) and hidden unit; rows: column k
    bool live;
};

// for the complex RBM, O_k = tanh(theta_j) (k < M) or s_i tanh(theta_j) (k = M + i M + j)
// (Psi.hpp:165-178)
__device__ __forceinline__ SmElem sm_elem_of(const SmSource& a, int k) {
    SmElem e{-1, k, k < a.L};
    if (a.kind == 0 && e.live && k >= a.M) {
        const int r = k - a.M;
        e.i = r / a.M;
        e.j = r - e.i * a.M;
    }
    return e;
}

// sqrt(w_s) (F[s][k] - shift[k]) (weight 1 unweighted), zero outside the matrix; the
// shift is subtracted in FP64 so that a centred matrix keeps the rows' small spread
__device__ __forceinline__ float2 sm_load_f(const SmSource& a, const SmElem& e, int s, int k) {
    if (!e.live || s >= a.count) return make_float2(0.0f, 0.0f);
    double2 d;
    if (a.kind == 0) {
        const float2 t = a.T[static_cast<long>(s) * a.Mpad + e.j];
        d = make_double2(t.x, t.y);
        if (e.i >= 0) {
            const uint64_t word = a.enumerate ? ((e.i >> 6) == 0 ? a.enum_base + static_cast<uint64_t>(s) : 0ull)
                                              : a.spins[static_cast<long>(s) * a.nw + (e.i >> 6)];
            if (!((word >> (e.i & 63)) & 1ull)) d = make_double2(-d.x, -d.y);
        }
    } else {
        d = a.rows[static_cast<long>(s) * a.ld + e.j];
    }
    if (a.shift) {
        d.x -= a.shift[k].x;
        d.y -= a.shift[k].y;
    }
    float2 v = make_float2(static_cast<float>(d.x), static_cast<float>(d.y));
    if (a.weighted) {
        const float c = static_cast<float>(sqrt(a.w[s]));
        v.x *= c;
        v.y *= c;
    }
    return v;
}

}  // namespace rbmg
