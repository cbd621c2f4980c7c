// Oracle (test infrastructure only): AC small-signal sweep restated from the
// reference.
//   frequency loop, ground row          crates/sim-core/src/engine.rs:829-930
//   complex MNA builder                 crates/sim-core/src/complex_mna.rs:1-181
//   AC stamps (R, C, V, I, D, M)        crates/sim-core/src/stamp.rs:1525-1750
//   dense complex LU, partial pivoting  crates/sim-core/src/complex_solver.rs:28-144
// Complex arithmetic is that of the num-complex crate (0.4.6, a dependency of
// sim-core that is not in the reference tree): a*b = (ar br - ai bi, ar bi +
// ai br); a/b = ((ar br + ai bi) / n, (ai br - ar bi) / n) with n = br br +
// bi bi; |a| = hypot(ar, ai); from_polar(r, t) = (r cos t, r sin t).
#include <algorithm>
#include <cmath>

#include "oracle.h"

namespace oracle {

namespace {
struct Cx {
  double re, im;
};
inline Cx cadd(Cx a, Cx b) { return {a.re + b.re, a.im + b.im}; }
inline Cx csub(Cx a, Cx b) { return {a.re - b.re, a.im - b.im}; }
inline Cx cmul(Cx a, Cx b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
inline Cx cdiv(Cx a, Cx b) {
  const double n = b.re * b.re + b.im * b.im;
  const double re = a.re * b.re + a.im * b.im;
  const double im = a.im * b.re - a.re * b.im;
  return {re / n, im / n};
}
inline double cnorm(Cx a) { return std::hypot(a.re, a.im); }
inline double xget(const Vec& x, size_t i) { return i < x.size() ? x[i] : 0.0; }

// ComplexSparseBuilder + ComplexStampContext
struct CBuilder {
  size_t n;
  std::vector<std::vector<std::pair<size_t, Cx>>> cols;
  std::vector<Cx> rhs;
  size_t node_count, naux = 0;
  explicit CBuilder(size_t nc) : n(nc), cols(nc), rhs(nc, Cx{0.0, 0.0}), node_count(nc) {}
  void add(size_t i, size_t j, Cx v) {  // insert(col = j, row = i), complex_mna.rs:18-23
    if (j >= n) return;
    cols[j].push_back({i, v});
  }
  void add_real(size_t i, size_t j, double v) { add(i, j, Cx{v, 0.0}); }
  void add_imag(size_t i, size_t j, double v) { add(i, j, Cx{0.0, v}); }
  void add_rhs(size_t i, Cx v) {
    if (i < rhs.size()) rhs[i] = cadd(rhs[i], v);
  }
  size_t allocate_aux() {  // every voltage source has its own name
    const size_t k = node_count + naux++;
    if (k + 1 > n) {
      cols.resize(k + 1);
      n = k + 1;
    }
    rhs.resize(n, Cx{0.0, 0.0});
    return k;
  }
};

Cx from_polar(double r, double deg) {
  const double t = deg * M_PI / 180.0;
  return {r * std::cos(t), r * std::sin(t)};
}
}  // namespace

// AC solution at every frequency: x[f * n + i] (n = nodes + one aux per V
// source). Returns 0, or 1 when a pivot's magnitude is below 1e-30.
int ac_sweep(const Circuit& c, const Vec& xdc, const Vec& freqs, std::vector<double>& out_re,
             std::vector<double>& out_im, size_t& n_out) {
  const double gmin = 1e-12;
  for (size_t fi = 0; fi < freqs.size(); ++fi) {
    const double omega = 2.0 * M_PI * freqs[fi];
    CBuilder b(c.node_count);
    for (size_t d = 0; d < c.ndev(); ++d) {
      const int32_t* nd = &c.nodes[d * 4];
      const double* p = &c.p[d * NPARAM];
      const size_t a = (size_t)nd[0], bb = (size_t)nd[1];
      switch (c.type[d]) {
        case DEV_R: {  // stamp.rs:1525-1543
          const double g = 1.0 / p[0];
          b.add_real(a, a, g);
          b.add_real(bb, bb, g);
          b.add_real(a, bb, -g);
          b.add_real(bb, a, -g);
          break;
        }
        case DEV_C: {  // stamp.rs:1545-1564
          const double y = omega * p[0];
          b.add_imag(a, a, y);
          b.add_imag(bb, bb, y);
          b.add_imag(a, bb, -y);
          b.add_imag(bb, a, -y);
          break;
        }
        case DEV_V: {  // stamp.rs:1594-1621; p1 = AC magnitude, p2 = phase [deg]
          const size_t k = b.allocate_aux();
          b.add_real(a, k, 1.0);
          b.add_real(bb, k, -1.0);
          b.add_real(k, a, 1.0);
          b.add_real(k, bb, -1.0);
          b.add_rhs(k, from_polar(p[1], p[2]));
          break;
        }
        case DEV_I: {  // stamp.rs:1623-1642
          const Cx i = from_polar(p[1], p[2]);
          b.add_rhs(a, Cx{-i.re, -i.im});
          b.add_rhs(bb, i);
          break;
        }
        case DEV_D: {  // stamp.rs:1644-1676, at the DC solution
          const double vt = 0.02585 * p[1];
          const double vd = xget(xdc, a) - xget(xdc, bb);
          const double gd = (p[0] / vt) * std::exp(vd / vt);
          const double g = std::fmax(gd, gmin);
          b.add_real(a, a, g);
          b.add_real(bb, bb, g);
          b.add_real(a, bb, -g);
          b.add_real(bb, a, -g);
          break;
        }
        case DEV_M: {  // stamp.rs:1678-1747 (level 1: gmbs = 0, not stamped)
          const size_t dr = (size_t)nd[0], gt = (size_t)nd[1], sr = (size_t)nd[2];
          const MosOut o = eval_level1(p[1], p[2], p[3], p[4], p[5], xget(xdc, dr),
                                       xget(xdc, gt), xget(xdc, sr), p[0] != 0.0);
          const double gm = o.gm, gds = std::fmax(o.gds, gmin);
          b.add_real(dr, dr, gds);
          b.add_real(sr, sr, gds);
          b.add_real(dr, sr, -gds);
          b.add_real(sr, dr, -gds);
          b.add_real(dr, gt, gm);
          b.add_real(dr, sr, -gm);
          b.add_real(sr, gt, -gm);
          b.add_real(sr, sr, gm);
          break;
        }
        case DEV_MC: {  // the consistent level 1: its exact small-signal Jacobian
          const size_t dr = (size_t)nd[0], gt = (size_t)nd[1], sr = (size_t)nd[2];
          const MosJ j = eval_level1_consistent(p[1], p[2], p[3], p[4], p[5], xget(xdc, dr),
                                                xget(xdc, gt), xget(xdc, sr), p[0] != 0.0,
                                                gmin);
          b.add_real(dr, dr, j.ddd);
          b.add_real(sr, sr, -j.dds);
          b.add_real(dr, sr, j.dds);
          b.add_real(sr, dr, -j.ddd);
          b.add_real(dr, gt, j.ddg);
          b.add_real(sr, gt, -j.ddg);
          break;
        }
        default:
          break;
      }
    }
    // ground: drop row 0, then (0,0) = 1 and rhs[0] = 0 (engine.rs:892-902)
    for (auto& col : b.cols)
      col.erase(std::remove_if(col.begin(), col.end(),
                               [](const std::pair<size_t, Cx>& e) { return e.first == 0; }),
                col.end());
    b.add(0, 0, Cx{1.0, 0.0});
    b.rhs[0] = Cx{0.0, 0.0};
    const size_t n = b.n;
    // finalize (stable sort by row) and the dense fill, duplicates added in
    // CSC order (complex_mna.rs:40-59, complex_solver.rs:70-79)
    std::vector<Cx> A(n * n, Cx{0.0, 0.0});
    for (size_t col = 0; col < n; ++col) {
      auto& e = b.cols[col];
      std::stable_sort(e.begin(), e.end(),
                       [](const std::pair<size_t, Cx>& x, const std::pair<size_t, Cx>& y) {
                         return x.first < y.first;
                       });
      for (auto& q : e) A[q.first * n + col] = cadd(A[q.first * n + col], q.second);
    }
    std::vector<Cx> x(b.rhs);
    for (size_t k = 0; k < n; ++k) {  // complex_solver.rs:84-120
      double mx = cnorm(A[k * n + k]);
      size_t mr = k;
      for (size_t i = k + 1; i < n; ++i) {
        const double v = cnorm(A[i * n + k]);
        if (v > mx) {
          mx = v;
          mr = i;
        }
      }
      if (mr != k) {
        for (size_t j = 0; j < n; ++j) std::swap(A[k * n + j], A[mr * n + j]);
        std::swap(x[k], x[mr]);
      }
      const Cx piv = A[k * n + k];
      if (cnorm(piv) < 1e-30) return 1;
      for (size_t i = k + 1; i < n; ++i) {
        const Cx f = cdiv(A[i * n + k], piv);
        A[i * n + k] = f;
        for (size_t j = k + 1; j < n; ++j) A[i * n + j] = csub(A[i * n + j], cmul(f, A[k * n + j]));
        x[i] = csub(x[i], cmul(f, x[k]));
      }
    }
    for (size_t ii = n; ii-- > 0;) {  // complex_solver.rs:122-133
      for (size_t j = ii + 1; j < n; ++j) x[ii] = csub(x[ii], cmul(A[ii * n + j], x[j]));
      const Cx piv = A[ii * n + ii];
      if (cnorm(piv) < 1e-30) return 1;
      x[ii] = cdiv(x[ii], piv);
    }
    if (fi == 0) {
      n_out = n;
      out_re.assign(freqs.size() * n, 0.0);
      out_im.assign(freqs.size() * n, 0.0);
    }
    for (size_t i = 0; i < n; ++i) {
      out_re[fi * n + i] = x[i].re;
      out_im[fi * n + i] = x[i].im;
    }
  }
  return 0;
}

}  // namespace oracle
