// Host-side check of the contraction descriptors of ttals_desc.cuh: every
// descriptor is evaluated on random data with the same offset/sum code the
// kernels use, compared with a naive loop nest, and every operand/output
// offset is checked against its buffer size.  Exit status 0 = all good.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <random>
#include <vector>

#include "ttals_desc.cuh"

using namespace ttals;
static std::mt19937_64 rng(7);
static std::vector<double> rnd(size_t n) {
  std::normal_distribution<double> d;
  std::vector<double> v(n);
  for (auto& x : v) x = d(rng);
  return v;
}
static int fails = 0;
static std::vector<double> run(const Contraction& c, const std::vector<double>& A, const std::vector<double>& B,
                               size_t csize) {
  std::vector<double> C(csize, NAN);
  for (int64_t e = 0; e < c.total; ++e) {
    int64_t ao, bo, co;
    contract_offsets(c, e, ao, bo, co);
    // bounds of every operand access
    int64_t amax = ao, bmax = bo;
    for (int q = 0; q < c.nk; ++q) {
      amax += (c.k_dim[q] - 1) * c.a_ks[q];
      bmax += (c.k_dim[q] - 1) * c.b_ks[q];
    }
    if (ao < 0 || bo < 0 || co < 0 || amax >= (int64_t)A.size() || bmax >= (int64_t)B.size() ||
        co >= (int64_t)csize) {
      std::printf("out of bounds: e=%lld a[%lld..%lld]/%zu b[%lld..%lld]/%zu c[%lld]/%zu\n", (long long)e,
                  (long long)ao, (long long)amax, A.size(), (long long)bo, (long long)bmax, B.size(), (long long)co,
                  csize);
      ++fails;
      return C;
    }
    C[co] = contract_sum(c, A.data(), B.data(), ao, bo);
  }
  return C;
}
static void expect(const char* what, const std::vector<double>& got, const std::vector<double>& ref) {
  double err = 0, mx = 0;
  for (size_t i = 0; i < ref.size(); ++i) {
    err = std::fmax(err, std::fabs(got[i] - ref[i]));
    mx = std::fmax(mx, std::fabs(ref[i]));
    if (std::isnan(got[i])) err = INFINITY;
  }
  if (!(err <= 1e-12 * (1 + mx))) {
    std::printf("%s: max err %g\n", what, err);
    ++fails;
  }
}

static void check_fast_div() {
  std::uniform_int_distribution<uint32_t> dn(0, (1u << 31) - 1);
  for (uint32_t d = 1; d < 5000; ++d) {
    uint32_t mag;
    int shf;
    fast_div_params(d, &mag, &shf);
    for (int t = 0; t < 200; ++t) {
      const uint32_t n = (t < 100) ? (uint32_t)t * 37u : dn(rng);
      if (fast_div(n, mag, shf) != n / d) {
        std::printf("fast_div wrong: %u / %u\n", n, d);
        ++fails;
        return;
      }
    }
  }
  for (uint32_t d : {65536u, 1u << 20, (1u << 30) + 7, (1u << 31) - 1}) {
    uint32_t mag;
    int shf;
    fast_div_params(d, &mag, &shf);
    for (uint32_t n : {0u, 1u, d - 1, d, d + 1, (1u << 31) - 1})
      if (fast_div(n, mag, shf) != n / d) {
        std::printf("fast_div wrong: %u / %u\n", n, d);
        ++fails;
      }
  }
}

int main() {
  check_fast_div();
  const int64_t shapes[][7] = {{3, 2, 4, 2, 3, 2, 3}, {5, 3, 2, 1, 4, 3, 1}, {1, 4, 6, 3, 1, 1, 2}, {4, 1, 4, 2, 2, 2, 2}};
  for (auto& sh : shapes) {
    const int64_t a = sh[0], n = sh[1], s = sh[2], R0 = sh[3], R1 = sh[4], h = sh[5], g = sh[6];
    auto L = rnd(a * R0 * a), A = rnd(R0 * n * n * R1), Rt = rnd(s * R1 * s), y = rnd(a * n * s);
    // apply
    Contraction p1, p2, p3;
    desc_apply(a, n, s, R0, R1, &p1, &p2, &p3);
    auto T1 = run(p1, L, y, R0 * a * n * s);
    auto T2 = run(p2, T1, A, a * n * s * R1);
    auto out = run(p3, T2, Rt, a * n * s);
    std::vector<double> ref(a * n * s, 0.0);
    for (int64_t ap = 0; ap < a; ++ap)
      for (int64_t m = 0; m < n; ++m)
        for (int64_t sp = 0; sp < s; ++sp) {
          double acc = 0;
          for (int64_t aa = 0; aa < a; ++aa)
            for (int64_t R = 0; R < R0; ++R)
              for (int64_t nn = 0; nn < n; ++nn)
                for (int64_t Q = 0; Q < R1; ++Q)
                  for (int64_t ss = 0; ss < s; ++ss)
                    acc += L[(aa * R0 + R) * a + ap] * A[((R * n + m) * n + nn) * R1 + Q] * Rt[(ss * R1 + Q) * s + sp] *
                           y[(aa * n + nn) * s + ss];
          ref[(ap * n + m) * s + sp] = acc;
        }
    expect("apply", out, ref);
    // left stack: L_new[s,Q,s'] = sum L[a,R,a'] x[a,n,s] A[R,m,n,Q] x[a',m,s']
    auto Ln = run(desc_left_p3(a, n, s, R1), T2, y, s * R1 * s);
    std::vector<double> rl(s * R1 * s, 0.0);
    for (int64_t s1 = 0; s1 < s; ++s1)
      for (int64_t Q = 0; Q < R1; ++Q)
        for (int64_t s2 = 0; s2 < s; ++s2) {
          double acc = 0;
          for (int64_t aa = 0; aa < a; ++aa)
            for (int64_t R = 0; R < R0; ++R)
              for (int64_t ap = 0; ap < a; ++ap)
                for (int64_t nn = 0; nn < n; ++nn)
                  for (int64_t m = 0; m < n; ++m)
                    acc += L[(aa * R0 + R) * a + ap] * y[(aa * n + nn) * s + s1] * A[((R * n + m) * n + nn) * R1 + Q] *
                           y[(ap * n + m) * s + s2];
          rl[(s1 * R1 + Q) * s + s2] = acc;
        }
    expect("left stack", Ln, rl);
    // right stack from Rn[s,Q,s']
    auto Rn = rnd(s * R1 * s);
    Contraction q1, q2, q3;
    desc_right(a, n, s, R0, R1, &q1, &q2, &q3);
    auto U1 = run(q1, Rn, y, s * R1 * a * n);
    auto U2 = run(q2, U1, A, s * R0 * n * a);
    auto Rr = run(q3, y, U2, a * R0 * a);
    std::vector<double> rr(a * R0 * a, 0.0);
    for (int64_t aa = 0; aa < a; ++aa)
      for (int64_t R = 0; R < R0; ++R)
        for (int64_t ap = 0; ap < a; ++ap) {
          double acc = 0;
          for (int64_t nn = 0; nn < n; ++nn)
            for (int64_t ss = 0; ss < s; ++ss)
              for (int64_t m = 0; m < n; ++m)
                for (int64_t Q = 0; Q < R1; ++Q)
                  for (int64_t s2 = 0; s2 < s; ++s2)
                    acc += y[(aa * n + nn) * s + ss] * A[((R * n + m) * n + nn) * R1 + Q] * y[(ap * n + m) * s + s2] *
                           Rn[(ss * R1 + Q) * s + s2];
          rr[(aa * R0 + R) * a + ap] = acc;
        }
    expect("right stack", Rr, rr);
    // vector stacks and local rhs
    auto Lb = rnd(h * a), b = rnd(h * n * g), Rb = rnd(g * s);
    auto U = run(desc_vec_u_left(a, n, h, g), Lb, b, a * n * g);
    auto Lbn = run(desc_vec_left(a, n, s, g), U, y, g * s);
    auto f = run(desc_micro_f(a, n, s, g), U, Rb, a * n * s);
    std::vector<double> rlb(g * s, 0.0), rf(a * n * s, 0.0);
    for (int64_t gg = 0; gg < g; ++gg)
      for (int64_t sp = 0; sp < s; ++sp)
        for (int64_t hh = 0; hh < h; ++hh)
          for (int64_t ap = 0; ap < a; ++ap)
            for (int64_t m = 0; m < n; ++m) rlb[gg * s + sp] += Lb[hh * a + ap] * b[(hh * n + m) * g + gg] * y[(ap * n + m) * s + sp];
    for (int64_t ap = 0; ap < a; ++ap)
      for (int64_t m = 0; m < n; ++m)
        for (int64_t sp = 0; sp < s; ++sp)
          for (int64_t hh = 0; hh < h; ++hh)
            for (int64_t gg = 0; gg < g; ++gg) rf[(ap * n + m) * s + sp] += Lb[hh * a + ap] * b[(hh * n + m) * g + gg] * Rb[gg * s + sp];
    expect("left vec", Lbn, rlb);
    expect("local rhs", f, rf);
    auto h2 = h;  // right vector stack from core x (a, n, s), b (h, n, g)
    auto Rbv = rnd(g * s);
    auto Ur = run(desc_vec_u_right(a, n, s, g), y, Rbv, a * n * g);
    auto Rbn = run(desc_vec_right(a, n, h2, g), b, Ur, h2 * a);
    std::vector<double> rrb(h2 * a, 0.0);
    for (int64_t hh = 0; hh < h2; ++hh)
      for (int64_t ap = 0; ap < a; ++ap)
        for (int64_t m = 0; m < n; ++m)
          for (int64_t gg = 0; gg < g; ++gg)
            for (int64_t sp = 0; sp < s; ++sp) rrb[hh * a + ap] += b[(hh * n + m) * g + gg] * y[(ap * n + m) * s + sp] * Rbv[gg * s + sp];
    expect("right vec", Rbn, rrb);
    // pushes
    auto X = rnd(7 * a), Rm = rnd(a * 3);
    auto pr = run(desc_push_right(7, a, 3), X, Rm, 21);
    std::vector<double> rpr(21, 0.0);
    for (int i = 0; i < 7; ++i)
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < a; ++k) rpr[i * 3 + j] += X[i * a + k] * Rm[k * 3 + j];
    expect("push right", pr, rpr);
    auto Rl = rnd(3 * s), Xs = rnd(s * 5);
    auto pl = run(desc_push_left(3, s, 5), Rl, Xs, 15);
    std::vector<double> rpl(15, 0.0);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 5; ++j)
        for (int k = 0; k < s; ++k) rpl[i * 5 + j] += Rl[i * s + k] * Xs[k * 5 + j];
    expect("push left", pl, rpl);
  }
  std::printf(fails ? "FAIL %d\n" : "OK\n", fails);
  return fails ? 1 : 0;
}
