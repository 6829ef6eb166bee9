// Contraction descriptors of the ALS hot path, usable from host and device.
//
// Every contraction is "one output element per thread": the output index space
// is row-major over up to 6 axes and each output sums a product over up to 3
// contraction axes; each axis carries its stride in both operands (and in the
// output).  Shapes (square local problem):
//   a = r_i, n = n_i, s = r_{i+1}, R0 = R_i, R1 = R_{i+1}, h/g = RHS ranks.
#pragma once

#include "ttals_device.cuh"

namespace ttals {

struct Ax {
  int64_t dim, sa, sb, sc;
};

__host__ __device__ inline Contraction desc_make(int nout, const Ax* out, int nk, const Ax* k) {
  Contraction c{};
  c.nout = nout;
  c.nk = nk;
  c.total = 1;
  for (int q = 0; q < nout; ++q) {
    c.out_dim[q] = (int)out[q].dim;
    fast_div_params((uint32_t)out[q].dim, &c.out_mag[q], &c.out_shf[q]);
    c.a_os[q] = (int)out[q].sa;
    c.b_os[q] = (int)out[q].sb;
    c.c_os[q] = (int)out[q].sc;
    c.total *= out[q].dim;
  }
  c.ktotal = 1;
  for (int q = 0; q < nk; ++q) {
    c.k_dim[q] = (int)k[q].dim;
    c.a_ks[q] = (int)k[q].sa;
    c.b_ks[q] = (int)k[q].sb;
    c.ktotal *= k[q].dim;
  }
  return c;
}

// y -> M y:  P1 T1[R,a',n,s] = sum_a L[a,R,a'] y[a,n,s]
//            P2 T2[a',m,s,Q] = sum_{R,n} T1[R,a',n,s] A[R,m,n,Q]
//            P3 out[a',m,s'] = sum_{s,Q} T2[a',m,s,Q] Rt[s,Q,s']
__host__ __device__ inline void desc_apply(int64_t a, int64_t n, int64_t s, int64_t R0, int64_t R1,
                                           Contraction* p1, Contraction* p2, Contraction* p3) {
  const Ax o1[4] = {{R0, a, 0, a * n * s}, {a, 1, 0, n * s}, {n, 0, s, s}, {s, 0, 1, 1}};
  const Ax k1[1] = {{a, R0 * a, n * s, 0}};
  *p1 = desc_make(4, o1, 1, k1);
  const Ax o2[4] = {{a, n * s, 0, n * s * R1}, {n, 0, n * R1, s * R1}, {s, 1, 0, R1}, {R1, 0, 1, 1}};
  const Ax k2[2] = {{R0, a * n * s, n * n * R1, 0}, {n, s, R1, 0}};
  *p2 = desc_make(4, o2, 2, k2);
  const Ax o3[3] = {{a, n * s * R1, 0, n * s}, {n, s * R1, 0, s}, {s, 0, 1, 1}};
  const Ax k3[2] = {{s, R1, R1 * s, 0}, {R1, 1, s, 0}};
  *p3 = desc_make(3, o3, 2, k3);
}

// left operator stack, last phase: L_new[s,Q,s'] = sum_{a',m} T2[a',m,s,Q] x[a',m,s']
__host__ __device__ inline Contraction desc_left_p3(int64_t a, int64_t n, int64_t s, int64_t Q) {
  const Ax o[3] = {{s, Q, 0, Q * s}, {Q, 1, 0, s}, {s, 0, 1, 1}};
  const Ax k[2] = {{a, n * s * Q, n * s, 0}, {n, s * Q, s, 0}};
  return desc_make(3, o, 2, k);
}

// right operator stack from Rn[s,Q,s'], core x[a,n,s], A[R,n,n,Q]:
//   Q1 U1[s,Q,a',m] = sum_s' Rn[s,Q,s'] x[a',m,s']
//   Q2 U2[s,R,n,a'] = sum_{Q,m} U1[s,Q,a',m] A[R,m,n,Q]
//   Q3 Rt[a,R,a']   = sum_{n,s} x[a,n,s] U2[s,R,n,a']
__host__ __device__ inline void desc_right(int64_t a, int64_t n, int64_t s, int64_t R, int64_t Q, Contraction* q1,
                                           Contraction* q2, Contraction* q3) {
  const Ax o1[4] = {{s, Q * s, 0, Q * a * n}, {Q, s, 0, a * n}, {a, 0, n * s, n}, {n, 0, s, 1}};
  const Ax k1[1] = {{s, 1, 1, 0}};
  *q1 = desc_make(4, o1, 1, k1);
  const Ax o2[4] = {{s, Q * a * n, 0, R * n * a}, {R, 0, n * n * Q, n * a}, {n, 0, Q, a}, {a, n, 0, 1}};
  const Ax k2[2] = {{Q, a * n, 1, 0}, {n, 1, n * Q, 0}};
  *q2 = desc_make(4, o2, 2, k2);
  const Ax o3[3] = {{a, n * s, 0, R * a}, {R, 0, n * a, a}, {a, 0, 1, 1}};
  const Ax k3[2] = {{n, s, a, 0}, {s, 1, R * n * a, 0}};
  *q3 = desc_make(3, o3, 2, k3);
}

// U[a',m,g] = sum_h Lb[h,a'] b[h,m,g]  (first half of the left vector stack and of the local rhs)
__host__ __device__ inline Contraction desc_vec_u_left(int64_t a, int64_t n, int64_t h, int64_t g) {
  const Ax o[3] = {{a, 1, 0, n * g}, {n, 0, g, g}, {g, 0, 1, 1}};
  const Ax k[1] = {{h, a, n * g, 0}};
  return desc_make(3, o, 1, k);
}
// Lb_new[g,s'] = sum_{a',m} U[a',m,g] x[a',m,s']
__host__ __device__ inline Contraction desc_vec_left(int64_t a, int64_t n, int64_t s, int64_t g) {
  const Ax o[2] = {{g, 1, 0, s}, {s, 0, 1, 1}};
  const Ax k[2] = {{a, n * g, n * s, 0}, {n, g, s, 0}};
  return desc_make(2, o, 2, k);
}
// U[a',m,g] = sum_s' x[a',m,s'] Rb[g,s']
__host__ __device__ inline Contraction desc_vec_u_right(int64_t a, int64_t n, int64_t s, int64_t g) {
  const Ax o[3] = {{a, n * s, 0, n * g}, {n, s, 0, g}, {g, 0, s, 1}};
  const Ax k[1] = {{s, 1, 1, 0}};
  return desc_make(3, o, 1, k);
}
// Rb_new[h,a'] = sum_{m,g} b[h,m,g] U[a',m,g]
__host__ __device__ inline Contraction desc_vec_right(int64_t a, int64_t n, int64_t h, int64_t g) {
  const Ax o[2] = {{h, n * g, 0, a}, {a, 0, n * g, 1}};
  const Ax k[2] = {{n, g, g, 0}, {g, 1, 1, 0}};
  return desc_make(2, o, 2, k);
}
// f[a',m,s'] = sum_g U[a',m,g] Rb[g,s']
__host__ __device__ inline Contraction desc_micro_f(int64_t a, int64_t n, int64_t s, int64_t g) {
  const Ax o[3] = {{a, n * g, 0, n * s}, {n, g, 0, s}, {s, 0, 1, 1}};
  const Ax k[1] = {{g, 1, s, 0}};
  return desc_make(3, o, 1, k);
}
// C (p x k) = X (p x a) * R (a x k)
__host__ __device__ inline Contraction desc_push_right(int64_t p, int64_t a, int64_t k) {
  const Ax o[2] = {{p, a, 0, k}, {k, 0, 1, 1}};
  const Ax kk[1] = {{a, 1, k, 0}};
  return desc_make(2, o, 1, kk);
}
// C (k x q) = R (k x s) * X (s x q)
__host__ __device__ inline Contraction desc_push_left(int64_t k, int64_t s, int64_t q) {
  const Ax o[2] = {{k, s, 0, q}, {q, 0, 1, 1}};
  const Ax kk[1] = {{s, 1, q, 0}};
  return desc_make(2, o, 1, kk);
}

}  // namespace ttals
