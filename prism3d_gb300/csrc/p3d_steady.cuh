// p3d_steady.cuh -- data layout of the steady-state driver.
#pragma once

#include "p3d_common.cuh"
#include "p3d_pe.cuh"

namespace p3d {

// Per-cell device arrays (structure of arrays, n cells each, C order of the
// grid).  Resident for the whole solve.
struct SteadyDev {
  // fixed by density (set at reset)
  const double* dens;
  double *g0, *av, *nh_col;
  int32_t* ray;
  double *ds, *kpd0, *uv0, *kci, *kco0, *hci0, *zeta, *td_rad;
  int8_t* fam;  // selected ray family: axis * 2 + (1 if cumsum ascends)
  // THEMIS grain state per cell (nano-grain fraction, band gap): the
  // reference's initial values at reset, then one grain step per dust step
  double *f_nano, *e_g;
  // state
  double *t_gas, *x_hi, *x_h2, *x_cp, *x_c, *x_co, *x_o, *x_e;
  // column layers of the current abundances, 2 n x_H2 and n x_CO (kept by
  // every kernel that writes x_H2 / x_CO), and the per-iteration columns
  double *l2, *l3;
  double *u_h2, *u_co;
  // per-cell outer T update memory
  double *t_prev, *r_prev, *t_lo, *t_hi, *span;
  // thermal root of the last iteration (warm start of the mixed path)
  double* t_root;
  // inputs at the last solve and the change it made (mixed-path compaction)
  double *u_h2_last, *u_co_last, *b_last, *chg_last;
  // cells solved this iteration (dense list) and values passed from the
  // chemistry kernel to the thermal kernel
  int32_t* list;
  // column tiles whose layers changed since their last column pass: x tiles
  // (j, k / 32), y tiles (i, k / 32), z pencils (i, j), one byte each
  uint8_t* col_dirty;
  // the worklist's per-cell tests, kept where their inputs are written:
  // q_self (thermal kernel) = last change <= quiet_tol and last thermal
  // residual <= quiet_r_tol; q_moved (column pass, cleared by the thermal
  // kernel) = a column moved by more than quiet_in_tol since the last solve
  uint8_t *q_self, *q_moved;
  double *rh2_cell, *chg_spec;
  // diagnostics of the last iteration
  double *fh2, *gamma_pe, *t_dust;
  int32_t* flags;
  // mixed thermal root: final node of the last full bisection (1024 + the
  // ten decisions as bits) and its smallest certified margin |net| / sum|terms|
  int16_t* bis_node;
  float* bis_margin;
  // |d ln f_H2 / d ln b| at the last chemistry solve (the worklist's test of
  // a Doppler-width drift)
  float* fh2_slope;
};

struct SteadyParams {
  double zeta0, x_c_total, x_o_total, x_hcop, t_init, f_nano, e_g;
  double sigma_nano, sigma_lc, sigma_sil;
  double w_chem, w_t, chem_rtol, therm_tol;
  double therm_tol_mixed;  // thermal-root tolerance of the mixed path
  double theta2;  // T_u of CO J = 1 (the ladder spacing 2 h B / k)
  int chem_max_iter, therm_max_iter, n_rays;
  int h2_implicit;  // 1: the cell's own H2 half layer is solved implicitly
  double count_thr[3];  // thresholds of the n_gt counters
  double quiet_tol;     // mixed path: skip cells whose last change was <= this
  double quiet_in_tol;  // ... and whose columns moved <= this since
  double quiet_b_tol;   // ... and whose H2 shielding factor moved <= this since
  double quiet_r_tol;   // ... and whose last thermal residual |G - T| / T was <= this
  // multipliers of the reduced network's rate coefficients (1 = the
  // reference's): H2 formation, H2 photodissociation, H2 cosmic-ray
  // destruction, C photoionisation, C+ recombination, CO photodissociation,
  // CR-induced CO dissociation, C + OH -> CO
  double rs[8];
  int fix_t;  // 1: T_gas is held at its current value (no thermal balance)
  int exact_roots;  // 1: mixed thermal roots to therm_tol_mixed even while a cell moves
  // mixed thermal kernel: lists of at most this many cells are solved one
  // cell per warp, the FP64 net heating evaluated by the whole warp
  int coop_max;
  PeGrid pe;
  LineParams lines;
  LineFast lf;  // make_line_fast(lines)
};

// Scalars shared between the kernels of one outer iteration.
struct SteadyGlobals {
  double t_mean, b_dop;
  unsigned long long dmax_bits;
  unsigned long long evals64;  // FP64 net-heating evaluations
  unsigned int chem_fail, therm_fail;
  unsigned int n_gt[3];  // cells with relative change > count_thr[k]
  unsigned int n_active;  // cells solved this iteration (length of the list)
  unsigned int therm_next;  // thermal kernel: next cell (mixed: list entry) to hand out
  unsigned int chem_next;   // chemistry kernel: the same
  int iter;
  int cols_all;  // 1: the next column pass recomputes every tile
};

// Columns of the per-iteration history record.
constexpr int kHistCols = 9;

}  // namespace p3d
