// p3d_adjoint.cuh -- adjoint of the steady state (implicit-function theorem).
//
// At the converged state every cell satisfies G_c(u_c, N_H2,c, N_CO,c, b; th)
// = 0 with u = (x_HI, x_H2, x_C+, x_C, x_CO, T): the five rows of the
// reduced chemistry (two rate equations, the C+ and CO equations, H and C
// conservation; p3d_newton.cuh) and the thermal balance net_heating(T) = 0
// with the context built from u (solver_3d.py:693-754).  The cells couple
// through the selected-ray columns N_H2 = ds (sum of upstream 2 n x_H2 +
// own half layer), N_CO (same with n x_CO) and through the Doppler parameter
// b of the grid-mean T (shielding.py:17-59).  For a loss L(u) the adjoint
//   J_c^T lam_c + (B^T lam)_c = dL/du_c
// (J_c the per-cell Jacobian including the cell's own half layers of N_H2 and
// N_CO, B the strictly-upstream column coupling and the mean-T coupling) is
// solved by block-Jacobi sweeps: per-cell 6x6 transposed solves plus a reverse scan of
// each ray family (suffix sums of ds dG/dN^T lam, the transpose of the
// forward column scan) and one grid sum for the mean T.  Then
//   dL/dth_k = -sum_c lam_c^T dG_c/dth_k.
// Parameters th: log multipliers of the eight reduced-network rate
// coefficients (SteadyParams::rs order) and log G0 (every G0-proportional
// per-cell quantity, the dust temperature and the PE heating follow).
//
// Local derivatives: the chemistry rows' derivatives with respect to the
// five abundances are chem5_eval's analytic Jacobian (p3d_newton.cuh); the
// thermal row, the T column and the derivatives with respect to the
// columns, b and the log parameters are central differences of the FP64
// residual with relative steps 1e-6 (state, columns, b) and 1e-6 absolute in
// log parameters.  Where
// the outer map T -> selected thermal root is discontinuous (the forward
// iteration converges onto the discontinuity) the thermal row is the
// condition that pins T there: a bisection decision of the root selection
// flipping (net heating zero at that midpoint, context at T), or a jump of
// the net heating itself (T held: dT = 0).
#pragma once

namespace p3d {

constexpr int kAdjParams = 9;
constexpr double kAdjStep = 1e-6;

struct AdjArgs {
  // per cell (n each unless stated)
  double* jinv;   // 36 n: inverse of the per-cell Jacobian, row-major
  double* jn2;    // 6 n: dG/dN_H2
  double* jn3;    // 6 n: dG/dN_CO
  double* jb;     // 6 n: dG/db
  double* jth;    // 6 kAdjParams n: dG/dth
  double* lam;    // 6 n
  double* cx2;    // n: coupling into x_H2
  double* cx3;    // n: coupling into x_CO
  double* a2;     // n: ds dG/dN_H2 . lam
  double* a3;     // n: ds dG/dN_CO . lam
  double* qb;     // n: dG/db . lam
  int* jump;      // n
  double* teval;  // n: thermal-row evaluation point (<= 0: T itself)
  double* dn;     // n: gradient with respect to log n_H
  double* red;    // reduction scratch (one value per block of the sums)
  double* scal;   // 2: qb total, a sum result
  unsigned long long* dmax;  // largest relative change of lam in the last sweep (bits)
  double w[6];    // loss weights: columns of x_HI, x_H2, x_C+, x_C, x_CO; mean T
};

// Per-cell residual G (6) at state u (6), columns n2, n3, Doppler b and log
// parameter offsets th (kAdjParams) -- the equations the forward kernels
// zero at the fixed point.
// Density-dependent inputs of a cell's residual: its own n_H and the ray-march
// results G0, A_V and N_H (selected ray) the per-cell constants derive from
// (ss_setup_kernel).
struct AdjStatic {
  double nh, g0, av, nhc;
};

__device__ __forceinline__ AdjStatic adj_static(const SteadyDev& d, int64_t i) {
  return AdjStatic{d.dens[i], d.g0[i], d.av[i], d.nh_col[i]};
}

__device__ void adj_residual(int64_t i, const SteadyDev& d, const SteadyParams& p,
                             const double* __restrict__ a_nano, const double* __restrict__ a_rest,
                             const double* u, double n2, double n3, double b, const double* th,
                             double t_eval, const AdjStatic& st, double* G,
                             double (*jchem)[5] = nullptr) {
  const double nh = st.nh;
  const double T = u[5];
  const double gs = exp(th[8]);
  double m[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) m[k] = p.rs[k] * exp(th[k]);
  const double av = st.av;
  const double g0 = st.g0 * gs;
  // per-cell constants as ss_setup_kernel forms them
  const double e374 = exp(-3.74 * av);
  const double kpd0 = 4.43e-11 * g0 * e374;
  const double uv0 = g0 * e374;
  const double kci = 2.56e-10 * g0 * exp(-3.02 * av);
  const double kco0 = 1.71e-10 * g0 * exp(-3.53 * av);
  const double hci0 = 3.0e-10 * g0 * exp(-3.0 * av);
  const double zeta = cr_rate(st.nhc, p.zeta0);
  const double xe = fmax(u[2] + p.x_hcop, 1e-30);
  const double td = tdust(tdust_rad(g0, av), nh, T);
  const double rh2 = h2_form(T, td, d.f_nano[i], p.sigma_nano, p.sigma_lc, p.sigma_sil);
  ChemCell cc;
  cc.n_h = nh;
  cc.kci = kci * m[3];
  cc.acp = 4.67e-12 * pow(T / 300.0, -0.6) * m[4];
  cc.rh2 = rh2 * nh * 0.5 * m[0];
  cc.rcr = 2.5 * zeta * 0.1 * m[2];
  cc.xc = p.x_c_total;
  cc.hcop = p.x_hcop;
  cc.kpd0 = kpd0 * m[1];
  cc.kco0 = kco0 * m[5];
  cc.kco_cr = 6.0 * zeta * m[6];
  cc.koh_s = m[7];
  cc.u_h2 = n2;
  cc.u_co = n3;
  cc.ds = 0.0;
  cc.b_dop = b;
  chem_prepare(cc);
  double f[5], J[5][5], sc[5], fh2;
  chem5_eval(cc, u, f, J, sc, &fh2);
#pragma unroll
  for (int k = 0; k < 5; ++k) G[k] = f[k];
  if (jchem)
#pragma unroll
    for (int r = 0; r < 5; ++r)
#pragma unroll
      for (int c = 0; c < 5; ++c) jchem[r][c] = J[r][c];
  const double x0 = u[0], x1 = u[1], x3 = u[3];
  ThermalCtx c;
  const double uv = uv0 * fh2;
  double gf = pe_cell(p.pe, a_nano, a_rest, g0, T, xe, nh, d.f_nano[i], d.e_g[i]);
  gf += 3.3e-11 * uv * x1 * nh * (0.4 * kEVtoErg);
  gf += rh2 * x0 * (nh * nh) * (1.5 * kEVtoErg);
  gf += 3.0e-10 * uv * x1 * nh * (2.0 * kEVtoErg) * (nh / (nh + 3e4));
  gf += zeta * (x0 + 2.0 * x1) * nh * (20.0 * kEVtoErg);
  gf += hci0 * x3 * nh * kEVtoErg;
  c.gamma_fixed = gf;
  const double mu = x1 > 0.5 ? 2.0 : 1.0;
  c.gg_coeff = 2.0 * 0.35 * 1e-21 * (nh * nh) * (mu == 2.0 ? kGgSpeedMu2 : kGgSpeedMu1) * kKBoltz;
  c.t_dust = td;
  c.n_e = xe * nh;
  c.n_hi = x0 * nh;
  c.n_h2 = x1 * nh;
  c.n_co = u[4] * nh;
  c.n_cp_nh = u[2] * nh;
  c.n_o_nh = fmax(p.x_o_total - u[4], 1e-30) * nh;
  c.n_c_nh = x3 * nh;
  G[5] = net_heating_fast64_body(t_eval > 0.0 ? t_eval : T, c, p.lf, c_co_ss, p.theta2);
}

// Gauss-Jordan inverse of a 6x6 matrix with partial pivoting; false if
// singular.
__device__ bool inv6(double (*A)[6], double (*X)[6]) {
#pragma unroll
  for (int r = 0; r < 6; ++r)
#pragma unroll
    for (int c = 0; c < 6; ++c) X[r][c] = r == c ? 1.0 : 0.0;
  for (int k = 0; k < 6; ++k) {
    int piv = k;
    double best = fabs(A[k][k]);
    for (int r = k + 1; r < 6; ++r)
      if (fabs(A[r][k]) > best) { best = fabs(A[r][k]); piv = r; }
    if (!(best > 0.0) || !isfinite(best)) return false;
    if (piv != k)
      for (int c = 0; c < 6; ++c) {
        double t = A[k][c]; A[k][c] = A[piv][c]; A[piv][c] = t;
        t = X[k][c]; X[k][c] = X[piv][c]; X[piv][c] = t;
      }
    const double inv = 1.0 / A[k][k];
    for (int c = 0; c < 6; ++c) { A[k][c] *= inv; X[k][c] *= inv; }
    for (int r = 0; r < 6; ++r) {
      if (r == k) continue;
      const double m = A[r][k];
      if (m == 0.0) continue;
      for (int c = 0; c < 6; ++c) { A[r][c] -= m * A[k][c]; X[r][c] -= m * X[k][c]; }
    }
  }
  return true;
}

// Local derivatives and the inverse Jacobian of every cell.
__global__ void __launch_bounds__(128)
adj_local_kernel(int64_t n, SteadyDev d, SteadyParams p, const double* __restrict__ a_nano,
                 const double* __restrict__ a_rest, double b, AdjArgs a, unsigned int* n_bad) {
  // p.fix_t: T is an input (no thermal balance), held like a jump cell
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double u[6] = {d.x_hi[i], d.x_h2[i], d.x_cp[i], d.x_c[i], d.x_co[i], d.t_gas[i]};
    const double n2 = d.u_h2[i], n3 = d.u_co[i];
    const AdjStatic st = adj_static(d, i);
    double th[kAdjParams];
#pragma unroll
    for (int k = 0; k < kAdjParams; ++k) th[k] = 0.0;
    double G0[6], Gp[6], Gm[6], Jc[5][5];
    adj_residual(i, d, p, a_nano, a_rest, u, n2, n3, b, th, -1.0, st, G0, Jc);
    // Thermal row.  A smooth root: net_heating(T) = 0.  Otherwise the outer
    // map T -> selected root is discontinuous at T: either the net heating
    // itself jumps there (T held: dT = 0), or one of the ten bisection
    // decisions of the root selection flips there -- then net_heating at
    // that bisection midpoint vanishes with the context taken at T, and that
    // is the row (t_eval = the midpoint).
    double t_eval = -1.0;
    bool jump = p.fix_t != 0;
    if (!jump) {
      const double hT = kAdjStep * u[5];
      double up[6], um[6];
      for (int q = 0; q < 6; ++q) { up[q] = u[q]; um[q] = u[q]; }
      up[5] += hT;
      um[5] -= hT;
      adj_residual(i, d, p, a_nano, a_rest, up, n2, n3, b, th, -1.0, st, Gp);
      adj_residual(i, d, p, a_nano, a_rest, um, n2, n3, b, th, -1.0, st, Gm);
      if (!(fabs(G0[5]) <= 0.05 * fabs(Gp[5] - Gm[5]))) {
        double lo = 10.0, hi = 1e5, best = INFINITY, t_best = -1.0, nmax = 0.0;
        double nk[10], tk[10];
        for (int k = 0; k < 10; ++k) {
          const double tm = sqrt(lo * hi);
          adj_residual(i, d, p, a_nano, a_rest, u, n2, n3, b, th, tm, st, Gp);
          nk[k] = Gp[5];
          tk[k] = tm;
          nmax = fmax(nmax, fabs(Gp[5]));
          if (Gp[5] > 0.0) lo = tm; else hi = tm;
        }
        for (int k = 0; k < 10; ++k)
          if (fabs(nk[k]) < best) { best = fabs(nk[k]); t_best = tk[k]; }
        if (best <= 1e-7 * nmax) t_eval = t_best;
        else jump = true;
      }
    }
    double J[6][6];
    for (int k = 0; k < 6; ++k) {
      const double h = kAdjStep * fmax(fabs(u[k]), 1e-300);
      double up[6], um[6];
      for (int q = 0; q < 6; ++q) { up[q] = u[q]; um[q] = u[q]; }
      up[k] += h;
      um[k] -= h;
      adj_residual(i, d, p, a_nano, a_rest, up, n2, n3, b, th, t_eval, st, Gp);
      adj_residual(i, d, p, a_nano, a_rest, um, n2, n3, b, th, t_eval, st, Gm);
      for (int r = 0; r < 6; ++r) J[r][k] = (Gp[r] - Gm[r]) / (2.0 * h);
    }
    // the chemistry block is exact: chem5_eval's analytic Jacobian (the
    // differences above supply the thermal row and the T column, which have
    // no closed form here)
    for (int r = 0; r < 5; ++r)
      for (int c = 0; c < 5; ++c) J[r][c] = Jc[r][c];
    // columns, Doppler parameter, log parameters
    double jn2[6], jn3[6], jb[6], jth[6 * kAdjParams];
    {
      const double h = kAdjStep * fmax(n2, 1e14);
      adj_residual(i, d, p, a_nano, a_rest, u, n2 + h, n3, b, th, t_eval, st, Gp);
      adj_residual(i, d, p, a_nano, a_rest, u, fmax(n2 - h, 0.0), n3, b, th, t_eval, st, Gm);
      const double w = h + fmin(h, n2);
      for (int r = 0; r < 6; ++r) jn2[r] = (Gp[r] - Gm[r]) / w;
    }
    {
      const double h = kAdjStep * fmax(n3, 1e10);
      adj_residual(i, d, p, a_nano, a_rest, u, n2, n3 + h, b, th, t_eval, st, Gp);
      adj_residual(i, d, p, a_nano, a_rest, u, n2, fmax(n3 - h, 0.0), b, th, t_eval, st, Gm);
      const double w = h + fmin(h, n3);
      for (int r = 0; r < 6; ++r) jn3[r] = (Gp[r] - Gm[r]) / w;
    }
    {
      const double h = kAdjStep * b;
      adj_residual(i, d, p, a_nano, a_rest, u, n2, n3, b + h, th, t_eval, st, Gp);
      adj_residual(i, d, p, a_nano, a_rest, u, n2, n3, b - h, th, t_eval, st, Gm);
      for (int r = 0; r < 6; ++r) jb[r] = (Gp[r] - Gm[r]) / (2.0 * h);
    }
    for (int k = 0; k < kAdjParams; ++k) {
      th[k] = kAdjStep;
      adj_residual(i, d, p, a_nano, a_rest, u, n2, n3, b, th, t_eval, st, Gp);
      th[k] = -kAdjStep;
      adj_residual(i, d, p, a_nano, a_rest, u, n2, n3, b, th, t_eval, st, Gm);
      th[k] = 0.0;
      for (int r = 0; r < 6; ++r) jth[r * kAdjParams + k] = (Gp[r] - Gm[r]) / (2.0 * kAdjStep);
    }
    // the cell's own half layers of N_H2 and N_CO enter its own Jacobian
    // (implicit), so the sweeps only carry the strictly-upstream coupling
    {
      const double dsn = d.ds[i] * d.dens[i];
      for (int r = 0; r < 6; ++r) {
        J[r][1] += jn2[r] * dsn;
        J[r][4] += jn3[r] * 0.5 * dsn;
      }
    }
    if (jump) {  // T held at the jump: thermal row dT = 0
      for (int c = 0; c < 6; ++c) J[5][c] = c == 5 ? 1.0 : 0.0;
      jn2[5] = jn3[5] = jb[5] = 0.0;
      for (int k = 0; k < kAdjParams; ++k) jth[5 * kAdjParams + k] = 0.0;
    }
    // equilibrate (columns by |u|, rows by their largest entry), invert,
    // undo: J^-1 = C (R J C)^-1 R
    double A[6][6], X[6][6], rs[6];
    for (int r = 0; r < 6; ++r) {
      double mx = 0.0;
      for (int c = 0; c < 6; ++c) {
        A[r][c] = J[r][c] * fmax(fabs(u[c]), 1e-300);
        mx = fmax(mx, fabs(A[r][c]));
      }
      rs[r] = mx > 0.0 ? 1.0 / mx : 1.0;
      for (int c = 0; c < 6; ++c) A[r][c] *= rs[r];
    }
    bool ok = inv6(A, X);
    double* ji = a.jinv + 36 * i;
    for (int r = 0; r < 6; ++r)
      for (int c = 0; c < 6; ++c)
        ji[6 * r + c] = ok ? fmax(fabs(u[r]), 1e-300) * X[r][c] * rs[c] : 0.0;
    if (!ok) atomicAdd(n_bad, 1u);
    for (int r = 0; r < 6; ++r) {
      a.jn2[6 * i + r] = jn2[r];
      a.jn3[6 * i + r] = jn3[r];
      a.jb[6 * i + r] = jb[r];
    }
    for (int q = 0; q < 6 * kAdjParams; ++q) a.jth[6 * kAdjParams * i + q] = jth[q];
    a.jump[i] = jump ? 1 : 0;
    a.teval[i] = t_eval;
  }
}

// dL/du of the loss sum_c n_c dx sum_s w_s x_s,c + w_t mean(T) (w: 5 species
// column weights then the mean-T weight, in AdjArgs::w).
__device__ __forceinline__ void adj_dldu(const SteadyDev& d, const double* w, int64_t i, int64_t n,
                                         double dx, double* g) {
  const double cn = d.dens[i] * dx;
#pragma unroll
  for (int k = 0; k < 5; ++k) g[k] = w[k] * cn;
  g[5] = w[5] / (double)n;
}

// Per-cell scalars of the coupling from the current lam.
__global__ void adj_couple_kernel(int64_t n, SteadyDev d, AdjArgs a) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double s2 = 0.0, s3 = 0.0, sb = 0.0;
    for (int r = 0; r < 6; ++r) {
      const double l = a.lam[6 * i + r];
      s2 += a.jn2[6 * i + r] * l;
      s3 += a.jn3[6 * i + r] * l;
      sb += a.jb[6 * i + r] * l;
    }
    const double ds = d.ds[i];
    a.a2[i] = ds * s2;
    a.a3[i] = ds * s3;
    a.qb[i] = sb;
    a.cx2[i] = 0.0;  // the own half layers are in the cell's Jacobian
    a.cx3[i] = 0.0;
  }
}

// Transpose of ss_columns_all_kernel: for each pencil and direction, cells
// upstream of a cell of that family receive its a2 / a3 (suffix sums).
__global__ void adj_scan_kernel(int axis, int64_t nx, int64_t ny, int64_t nz, int64_t n_pencils,
                                const double* __restrict__ dens, const int8_t* __restrict__ fam,
                                AdjArgs a) {
  int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= n_pencils) return;
  int64_t base, stride, len;
  if (axis == 0) { base = p; stride = ny * nz; len = nx; }
  else if (axis == 1) { int64_t i = p / nz, k = p - i * nz; base = i * ny * nz + k; stride = nz; len = ny; }
  else { base = p * nz; stride = 1; len = nz; }
  for (int fwd = 1; fwd >= 0; --fwd) {
    const int8_t want = (int8_t)(axis * 2 + fwd);
    double acc2 = 0.0, acc3 = 0.0;
    for (int64_t t = len - 1; t >= 0; --t) {  // reverse of the forward order
      const int64_t c = base + (fwd ? t : (len - 1 - t)) * stride;
      const double nc = dens[c];
      a.cx2[c] += 2.0 * nc * acc2;
      a.cx3[c] += nc * acc3;
      if (fam[c] == want) {
        acc2 += a.a2[c];
        acc3 += a.a3[c];
      }
    }
  }
}

// lam_c <- omega J_c^-T (dL/du_c - coupling_c) + (1 - omega) lam_c; records
// the largest relative change.
__global__ void adj_update_kernel(int64_t n, SteadyDev d, AdjArgs a, double dx,
                                  const double* __restrict__ qb_total, double dbdt,
                                  double omega) {
  double my = 0.0;
  const double qt = qb_total[0] * dbdt / (double)n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double g[6];
    adj_dldu(d, a.w, i, n, dx, g);
    g[1] -= a.cx2[i];
    g[4] -= a.cx3[i];
    g[5] -= qt;
    const double* ji = a.jinv + 36 * i;
    for (int c = 0; c < 6; ++c) {
      double l = 0.0;
      for (int r = 0; r < 6; ++r) l += ji[6 * r + c] * g[r];  // (J^-1)^T g
      const double old = a.lam[6 * i + c];
      const double nl = omega * l + (1.0 - omega) * old;
      my = fmax(my, fabs(nl - old) / fmax(fabs(nl), 1e-300));
      a.lam[6 * i + c] = nl;
    }
  }
  if (!(my == my)) my = INFINITY;
  block_max_atomic(my, a.dmax);
}

__global__ void adj_finish_sum_kernel(int nparts, const double* __restrict__ part,
                                      double* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0;
  for (int b = 0; b < nparts; ++b) s += part[b];
  out[0] = s;
}

// Per-cell contributions -lam_c . dG_c/dth_k into q (k-th parameter).
__global__ void adj_grad_kernel(int64_t n, AdjArgs a, int k, double* __restrict__ q) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int r = 0; r < 6; ++r) s += a.lam[6 * i + r] * a.jth[6 * kAdjParams * i + r * kAdjParams + k];
    q[i] = -s;
  }
}

// Gradient with respect to log n_H, local part: explicit loss term, the
// cell's own residual, and its layers in the N_H2 / N_CO columns of the
// cells downstream (cx2 / cx3 hold the strictly-upstream coupling of the
// final lam).  Also the scalars lam . dG/d(G0, A_V, N_H) the ray scans
// below need.
__global__ void __launch_bounds__(128)
adj_dens_local_kernel(int64_t n, SteadyDev d, SteadyParams p, const double* __restrict__ a_nano,
                      const double* __restrict__ a_rest, double b, double dx, AdjArgs a,
                      double* __restrict__ qg0, double* __restrict__ qav,
                      double* __restrict__ qnh) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double u[6] = {d.x_hi[i], d.x_h2[i], d.x_cp[i], d.x_c[i], d.x_co[i], d.t_gas[i]};
    const double n2 = d.u_h2[i], n3 = d.u_co[i];
    const double t_eval = a.teval[i];
    const bool held = a.jump[i] != 0;
    double th[kAdjParams];
    for (int k = 0; k < kAdjParams; ++k) th[k] = 0.0;
    double lam[6];
    for (int r = 0; r < 6; ++r) lam[r] = a.lam[6 * i + r];
    const AdjStatic st0 = adj_static(d, i);
    double q[4];
    for (int k = 0; k < 4; ++k) {
      AdjStatic sp = st0, sm = st0;
      double w;
      if (k == 0) { sp.nh = st0.nh * exp(kAdjStep); sm.nh = st0.nh * exp(-kAdjStep); w = 2.0 * kAdjStep; }
      else if (k == 1) { const double h = kAdjStep * st0.g0; sp.g0 += h; sm.g0 -= h; w = 2.0 * h; }
      else if (k == 2) { const double h = kAdjStep * fmax(st0.av, 1.0); sp.av += h; sm.av -= h; w = 2.0 * h; }
      else { const double h = kAdjStep * fmax(st0.nhc, 1e18); sp.nhc += h; sm.nhc = fmax(sm.nhc - h, 0.0); w = h + fmin(h, st0.nhc); }
      double Gp[6], Gm[6];
      adj_residual(i, d, p, a_nano, a_rest, u, n2, n3, b, th, t_eval, sp, Gp);
      adj_residual(i, d, p, a_nano, a_rest, u, n2, n3, b, th, t_eval, sm, Gm);
      double acc = 0.0;
      for (int r = 0; r < (held ? 5 : 6); ++r) acc += lam[r] * (Gp[r] - Gm[r]) / w;
      q[k] = acc;
    }
    double s2 = 0.0, s3 = 0.0;
    for (int r = 0; r < 6; ++r) {
      s2 += a.jn2[6 * i + r] * lam[r];
      s3 += a.jn3[6 * i + r] * lam[r];
    }
    const double nh = st0.nh, dsn = d.ds[i] * nh;
    double g = nh * dx * (a.w[0] * u[0] + a.w[1] * u[1] + a.w[2] * u[2] + a.w[3] * u[3] +
                          a.w[4] * u[4]);
    g -= q[0];
    g -= u[1] * (a.cx2[i] + s2 * dsn);
    g -= u[4] * (a.cx3[i] + 0.5 * s3 * dsn);
    a.dn[i] = g;
    qg0[i] = q[1];
    qav[i] = q[2];
    qnh[i] = q[3];
  }
}

// Gradient with respect to log n_H through the ray march: for ray r, every
// cell's G0 (if the ray carries external field) and, where r is the cell's
// selected ray, its A_V and N_H depend on the densities upstream along r.
// Reverse scan of the pencils of r's family: dn[c] -= n_c ds (sum over
// downstream c' of a(c') + a(c) / 2), a(c') = lam . dG/d(G0, A_V, N_H) times
// the derivative of those with respect to N_H,r(c').
__global__ void adj_ray_scan_kernel(int axis, int fwd, int ray, double ds, double gw,
                                    int64_t nx, int64_t ny, int64_t nz, int64_t n_pencils,
                                    const double* __restrict__ dens, const int32_t* __restrict__ sel,
                                    const double* __restrict__ qg0, const double* __restrict__ qav,
                                    const double* __restrict__ qnh, double* __restrict__ dn) {
  int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= n_pencils) return;
  int64_t base, stride, len;
  if (axis == 0) { base = p; stride = ny * nz; len = nx; }
  else if (axis == 1) { int64_t i = p / nz, k = p - i * nz; base = i * ny * nz + k; stride = nz; len = ny; }
  else { base = p * nz; stride = 1; len = nz; }
  double tot = 0.0;
  for (int64_t t = 0; t < len; ++t) tot += dens[base + t * stride];
  double suf = 0.0, acc = 0.0;
  for (int64_t t = len - 1; t >= 0; --t) {  // reverse of the forward order
    const int64_t c = base + (fwd ? t : (len - 1 - t)) * stride;
    const double nc = dens[c];
    const double nh_r = ds * (tot - suf - 0.5 * nc);  // upstream + own half layer
    double a_c = 0.0;
    if (nh_r > 0.0) {
      if (gw != 0.0) a_c += qg0[c] * gw * exp(-1.8 * nh_r * kAVperNH) * (-1.8 * kAVperNH);
      if (sel[c] == ray) a_c += qav[c] * kAVperNH + qnh[c];
    }
    dn[c] -= nc * ds * (acc + 0.5 * a_c);
    acc += a_c;
    suf += nc;
  }
}

__global__ void adj_jump_count_kernel(int64_t n, const int* __restrict__ jump,
                                      double* __restrict__ q) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    q[i] = (double)jump[i];
}

// Loss per cell: column part (weights w[0..4]) and T.
__global__ void adj_loss_kernel(int64_t n, SteadyDev d, AdjArgs a, double dx,
                                double* __restrict__ qcol, double* __restrict__ qt) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    qcol[i] = d.dens[i] * dx * (a.w[0] * d.x_hi[i] + a.w[1] * d.x_h2[i] + a.w[2] * d.x_cp[i] +
                                a.w[3] * d.x_c[i] + a.w[4] * d.x_co[i]);
    qt[i] = d.t_gas[i];
  }
}

}  // namespace p3d
