// Reverse sweep of one large step (the reverse mode the reference gets from torch autograd
// through atm_srk3(differentiable=True) with its per-step checkpoint,
// mpas_pytorch/autodiff/checkpoint.py:106-254, atmosphere_model.py:120-154).
//
// The caller restores the step's start state from its checkpoint; the step is then run
// forward once more while the values its reverse pass needs are kept in the tape: the state
// at the start of every RK stage (and at the end), the saves of every dynamics substep, every
// RK stage's tendencies, every implicit-coefficient set and every acoustic substep's inputs
// and outputs.  The saves, tendencies and coefficients are written into the tape by the
// forward kernels themselves (their field pointers point into the tape); the state and the
// acoustic fields are copied.  The stages then run backwards, each stage VJP reading its
// forward values from the tape.
#include <cmath>

#include "adj_common.cuh"

namespace {

#define CHECK_RC(x)                  \
  do {                               \
    int _rc = (x);                   \
    if (_rc != MPASG_OK) return _rc; \
  } while (0)

// the carried fields of a step boundary, in tape order
enum SnapField {
  S_U, S_V, S_RU, S_HEDGE, S_PVEDGE,            // edges
  S_W, S_RW,                                    // w levels
  S_THETA, S_RHOZZ, S_RHOP, S_RTHETAP, S_EXNER, S_PP, S_DIV, S_KE,  // cells
  S_VORT,                                       // vertices
  S_COUNT
};

double** snap_ptr(mpasg_fields& f, int k) {
  switch (k) {
    case S_U: return &f.u;
    case S_V: return &f.v;
    case S_RU: return &f.ru;
    case S_HEDGE: return &f.h_edge;
    case S_PVEDGE: return &f.pv_edge;
    case S_W: return &f.w;
    case S_RW: return &f.rw;
    case S_THETA: return &f.theta_m;
    case S_RHOZZ: return &f.rho_zz;
    case S_RHOP: return &f.rho_p;
    case S_RTHETAP: return &f.rtheta_p;
    case S_EXNER: return &f.exner;
    case S_PP: return &f.pressure_p;
    case S_DIV: return &f.divergence;
    case S_KE: return &f.ke;
    default: return &f.vorticity;
  }
}

struct StepPlan {
  int split, order, ns, nvimp_per_sub;
  double dt_dyn, rk_ts[3], rk_sub[3];
  int nsub[3];
  int n_ac;  // acoustic substeps per step
};

StepPlan plan_of(const mpasg_config* c) {
  StepPlan p{};
  p.split = c->dynamics_split_steps;
  p.order = c->time_integration_order;
  p.ns = c->number_of_sub_steps;
  p.dt_dyn = c->dt / p.split;
  const double d = p.dt_dyn;
  const int ns = p.ns;
  if (p.order == 3) {
    p.rk_ts[0] = d / 3.0; p.rk_ts[1] = d / 2.0; p.rk_ts[2] = d;
    p.rk_sub[0] = d / 3.0; p.rk_sub[1] = d / ns; p.rk_sub[2] = d / ns;
    p.nsub[0] = 1; p.nsub[1] = ns / 2 > 1 ? ns / 2 : 1; p.nsub[2] = ns;
  } else {
    p.rk_ts[0] = d / 2.0; p.rk_ts[1] = d / 2.0; p.rk_ts[2] = d;
    p.rk_sub[0] = p.rk_sub[1] = p.rk_sub[2] = d / ns;
    p.nsub[0] = p.nsub[1] = ns / 2 > 1 ? ns / 2 : 1; p.nsub[2] = ns;
  }
  p.nvimp_per_sub = p.order == 3 ? 2 : 1;
  p.n_ac = p.split * (p.nsub[0] + p.nsub[1] + p.nsub[2]);
  return p;
}

// Tape of the dynamics substeps lo..hi (1-based) of one step (doubles, every array rounded
// to 32 doubles): the carried fields at the start of every RK stage of the window and at
// its end, the window's substep saves, implicit-coefficient sets and acoustic-substep
// outputs.  Indices passed to the accessors are the step's own (stage i = 3 (sub-1) + rk-1,
// substep sub-1, coefficient slot, acoustic substep a); tendencies are not kept (the
// reverse pass reads none of their values).
struct Tape {
  long long E, W, C, V, Lr;
  long long snap_sz, sv_sz, coef_sz, aco_sz, sg_sz;
  int lo, hi, n_snap, n_sv, n_coef, n_ac, n_sg, per_sub_ac, nvimp;
  double* base = nullptr;
  Tape(const mpasg_mesh* m, const StepPlan& p, int lo_ = 1, int hi_ = 0) {
    const long long L = m->nVertLevels;
    lo = lo_;
    hi = hi_ > 0 ? hi_ : p.split;
    E = adj_round((m->nEdges + 1LL) * L);
    W = adj_round((m->nCells + 1LL) * (L + 1));
    C = adj_round((m->nCells + 1LL) * L);
    V = adj_round((m->nVertices + 1LL) * L);
    Lr = adj_round(L);
    snap_sz = 5 * E + 2 * W + 8 * C + V;
    sv_sz = E + W + 4 * C;
    coef_sz = Lr + 8 * C + W;
    aco_sz = E + 2 * W + 3 * C;
    // over terrain: the sign bytes of every RK stage's tend_u (the small-step slope terms'
    // selection)
    sg_sz = m->flatTerrain ? 0 : adj_round(((m->nEdges + 1LL) * L + 7) / 8);
    const int nsub = hi - lo + 1;
    nvimp = p.nvimp_per_sub;
    per_sub_ac = p.nsub[0] + p.nsub[1] + p.nsub[2];
    n_snap = 3 * nsub + 1;
    n_sv = nsub;
    n_coef = nsub * nvimp;
    n_ac = nsub * per_sub_ac;
    n_sg = sg_sz > 0 ? 3 * nsub : 0;
  }
  bool in(int sub) const { return sub >= lo && sub <= hi; }
  long long doubles() const {
    return n_snap * snap_sz + n_sv * sv_sz + n_coef * coef_sz + n_ac * aco_sz + n_sg * sg_sz;
  }
  // RK stage i's tend_u >= 0 bytes (terrain only)
  uint8_t* sg(int i) const {
    return reinterpret_cast<uint8_t*>(base + n_snap * snap_sz + n_sv * sv_sz + n_coef * coef_sz + n_ac * aco_sz +
                                      (i - 3 * (lo - 1)) * sg_sz);
  }
  double* snap(int i) const { return base + (i - 3 * (lo - 1)) * snap_sz; }
  double* sv(int i) const { return base + n_snap * snap_sz + (i - (lo - 1)) * sv_sz; }
  double* coef(int i) const { return base + n_snap * snap_sz + n_sv * sv_sz + (i - (lo - 1) * nvimp) * coef_sz; }
  // acoustic substep a: its outputs (ru_p after the edge update, the undamped solution x,
  // the damped solution rw_p, ts, rtheta_pp and rtheta_pp_old)
  double* aco(int a) const {
    return base + n_snap * snap_sz + n_sv * sv_sz + n_coef * coef_sz + (a - (lo - 1) * per_sub_ac) * aco_sz;
  }
  // the pointer of snapshot field k inside snapshot block b
  double* snap_field(double* b, int k) const {
    if (k < S_W) return b + k * E;
    if (k < S_THETA) return b + 5 * E + (k - S_W) * W;
    if (k < S_VORT) return b + 5 * E + 2 * W + (k - S_THETA) * C;
    return b + 5 * E + 2 * W + 8 * C;
  }
};

long long snap_len(const mpasg_mesh* m, int k) {
  const long long L = m->nVertLevels;
  if (k < S_W) return (m->nEdges + 1LL) * L;
  if (k < S_THETA) return (m->nCells + 1LL) * (L + 1);
  if (k < S_VORT) return (m->nCells + 1LL) * L;
  return (m->nVertices + 1LL) * L;
}

int dcopy(double* dst, const double* src, long long n, cudaStream_t s) {
  if (cudaMemcpyAsync(dst, src, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return MPASG_E_CUDA;
  return MPASG_OK;
}

// copy the carried fields of f into snapshot block b
int snap_store(const mpasg_mesh* m, const Tape& T, mpasg_fields& f, double* b, cudaStream_t s) {
  for (int k = 0; k < S_COUNT; ++k) CHECK_RC(dcopy(T.snap_field(b, k), *snap_ptr(f, k), snap_len(m, k), s));
  return MPASG_OK;
}

// copy the carried fields of snapshot block b back into the fields of f
int snap_restore(const mpasg_mesh* m, const Tape& T, mpasg_fields& f, const double* b, cudaStream_t s) {
  for (int k = 0; k < S_COUNT; ++k)
    CHECK_RC(dcopy(*snap_ptr(f, k), T.snap_field(const_cast<double*>(b), k), snap_len(m, k), s));
  return MPASG_OK;
}

// Up to S_COUNT (src, dst, offset, count) copies in one launch (blockIdx.y picks the copy).
struct CarryList {
  const double* src[S_COUNT];
  double* dst[S_COUNT];
  long long off[S_COUNT], n[S_COUNT];
};
__global__ void k_carry(CarryList cl) {
  const int j = blockIdx.y;
  const double* a = cl.src[j] + cl.off[j];
  double* b = cl.dst[j] + cl.off[j];
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < cl.n[j]; i += (long long)gridDim.x * blockDim.x)
    b[i] = a[i];
}

// What the recovery and the diagnostics of RK stage rk leave unwritten in the next snapshot
// block, carried over from this one: the padding rows of every carried field, the whole of
// rw (recovery writes its interior interfaces only), and before rk 3 the whole of exner and
// pressure_p (recovered at rk 3 only) and v (recomputed at rk 3 only).
int carry_block(const mpasg_mesh* m, const Tape& T, double* b0, double* b1, int rk, cudaStream_t s) {
  const long long L = m->nVertLevels;
  CarryList cl{};
  long long nmax = 0;
  for (int k = 0; k < S_COUNT; ++k) {
    const long long len = snap_len(m, k);
    const long long row = (k == S_W || k == S_RW) ? L + 1 : L;
    const bool whole = k == S_RW || (rk < 3 && (k == S_EXNER || k == S_PP || k == S_V));
    cl.src[k] = T.snap_field(b0, k);
    cl.dst[k] = T.snap_field(b1, k);
    cl.off[k] = whole ? 0 : len - row;
    cl.n[k] = whole ? len : row;
    if (cl.n[k] > nmax) nmax = cl.n[k];
  }
  long long gx = (nmax + kBlock - 1) / kBlock;
  if (gx > 1216) gx = 1216;
  k_carry<<<dim3((unsigned)gx, S_COUNT), kBlock, 0, s>>>(cl);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

// point the carried fields of v at snapshot block b
void snap_view(const Tape& T, mpasg_fields& v, double* b) {
  for (int k = 0; k < S_COUNT; ++k) *snap_ptr(v, k) = T.snap_field(b, k);
}

// saves of dynamics substep sub (0-based) in the tape
void sv_view(const Tape& T, mpasg_fields& v, int sub) {
  double* b = T.sv(sub);
  v.ru_save = b;
  v.rw_save = b + T.E;
  v.rtheta_p_save = b + T.E + T.W;
  v.rho_p_save = b + T.E + T.W + T.C;
  v.theta_m_save = b + T.E + T.W + 2 * T.C;
  v.rr_save = b + T.E + T.W + 3 * T.C;
}

void coef_view(const Tape& T, mpasg_fields& v, int j) {
  double* b = T.coef(j);
  v.cofrz = b;
  b += T.Lr;
  v.cofwr = b; b += T.C;
  v.cofwz = b; b += T.C;
  v.cofwt = b; b += T.C;
  v.a_tri = b; b += T.C;
  v.b_tri = b; b += T.C;
  v.c_tri = b; b += T.C;
  v.alpha_tri = b; b += T.C;
  v.gamma_tri = b; b += T.C;
  v.coftz = b;
}

// point the substep's scratch outputs (x, ts, rtheta_pp_old: written, not updated, by the
// substep) into its tape block, so they need no copy
void aco_redirect(const Tape& T, mpasg_fields& v, int a) {
  double* b = T.aco(a);
  v.ac_x = b + T.E;
  v.ac_ts = b + T.E + 2 * T.W;
  v.rtheta_pp_old = b + T.E + 2 * T.W + 2 * T.C;
}

// the substep's outputs the reverse pass reads (after the acoustic step, before damping)
// (the updated fields ru_p, rw_p and rtheta_pp are copied; x, ts and rtheta_pp_old were
// written there directly, aco_redirect)
int aco_store(const mpasg_mesh* m, const Tape& T, const mpasg_fields& f, int a, cudaStream_t s) {
  const long long L = m->nVertLevels;
  const long long nel = (m->nEdges + 1LL) * L, ncw = (m->nCells + 1LL) * (L + 1), ncl = (m->nCells + 1LL) * L;
  double* b = T.aco(a);
  CHECK_RC(dcopy(b, f.ru_p, nel, s));
  CHECK_RC(dcopy(b + T.E + T.W, f.rw_p, ncw, s));
  CHECK_RC(dcopy(b + T.E + 2 * T.W + T.C, f.rtheta_pp, ncl, s));
  return MPASG_OK;
}

// a view whose acoustic fields are substep a's taped outputs
void aco_view(const Tape& T, mpasg_fields& v, int a) {
  double* b = T.aco(a);
  v.ru_p = b;
  v.ac_x = b + T.E;
  v.rw_p = b + T.E + T.W;
  v.ac_ts = b + T.E + 2 * T.W;
  v.rtheta_pp = b + T.E + 2 * T.W + T.C;
  v.rtheta_pp_old = b + T.E + 2 * T.W + 2 * T.C;
}

__global__ void k_fill_row(double* __restrict__ p, int n, double v) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) p[i] = v;
}

__global__ void k_add2(double* __restrict__ y, double* __restrict__ x, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    y[i] = y[i] + x[i];
    x[i] = 0.0;
  }
}

// y += x, x = 0 (a save's cotangent returned to the state field it copied)
int fold(double* y, double* x, long long n, cudaStream_t s) {
  k_add2<<<nblocks(n), kBlock, 0, s>>>(y, x, n);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

// the edge-sum cotangent of theta_m_save (theta_edge_save = 0.5 (th_1 + th_2) and its
// reciprocal-sum partner) gathered on the cells: theta_m_save += sum over the cell's edges
__global__ void k_theta_edge_vjp(mpasg_mesh m, mpasg_fields g, FastDiv fl) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  const uint32_t c = fl.div(i);
  const int k = (int)(i - c * L);
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  double a = 0.0;
  for (int j = 0; j < n; ++j) a += g.theta_edge_save[(size_t)m.edgesOnCell[c * me + j] * L + k];
  g.theta_m_save[i] += a;
}

// the saves' cotangents returned to the state fields they copied (atm_rk_integration_setup
// and the substep refresh: ru_save = ru, rw_save = rw, rtheta_p_save = rtheta_p, rho_p_save =
// rr_save = rho_p, theta_m_save = theta_m)
int fold_saves(const mpasg_mesh* m, mpasg_fields* g, cudaStream_t s) {
  const long long L = m->nVertLevels;
  const long long nel = (m->nEdges + 1LL) * L, ncw = (m->nCells + 1LL) * (L + 1), ncl = (m->nCells + 1LL) * L;
  CHECK_RC(fold(g->ru, g->ru_save, nel, s));
  CHECK_RC(fold(g->rw, g->rw_save, ncw, s));
  CHECK_RC(fold(g->rtheta_p, g->rtheta_p_save, ncl, s));
  CHECK_RC(fold(g->rho_p, g->rho_p_save, ncl, s));
  CHECK_RC(fold(g->rho_p, g->rr_save, ncl, s));
  CHECK_RC(fold(g->theta_m, g->theta_m_save, ncl, s));
  return MPASG_OK;
}

// refresh the saves of the coming dynamics substep (writes go to the tape's save block);
// mixed: the mixed form's edge reciprocal sums, as its step forms them
int make_saves(const mpasg_mesh* m, const Tape& T, mpasg_fields& f, int sub, bool mixed, cudaStream_t s) {
  const long long L = m->nVertLevels, nc = m->nCells;
  const long long nel = (m->nEdges + 1LL) * L, ncw = (nc + 1) * (L + 1), ncl = (nc + 1) * L;
  k_fill_row<<<1, 128, 0, s>>>(f.theta_m + nc * L, (int)L, 0.0);
  MPASG_LAUNCH_CHECK();
  if (T.in(sub + 1)) sv_view(T, f, sub);
  CHECK_RC(dcopy(f.ru_save, f.ru, nel, s));
  CHECK_RC(dcopy(f.rw_save, f.rw, ncw, s));
  CHECK_RC(dcopy(f.rtheta_p_save, f.rtheta_p, ncl, s));
  CHECK_RC(dcopy(f.rho_p_save, f.rho_p, ncl, s));
  CHECK_RC(dcopy(f.theta_m_save, f.theta_m, ncl, s));
  CHECK_RC(dcopy(f.rr_save, f.rho_p, ncl, s));
  return mpasgi_theta_edge(m, &f, mixed, s);
}

int coef_slot(const StepPlan& p, int sub, int rk) {  // sub 1-based
  return (sub - 1) * p.nvimp_per_sub + ((rk == 1 || p.order == 2) ? 0 : 1);
}

// the step's dynamics forward with the tape (no transport, no reconstruction); in the
// mixed form the same stage calls as its step (float32 copies packed at the step start,
// kept current by the stages), so the values are that form's trajectory
// The step's dynamics forward (no transport, no reconstruction) up to the end of the tape's
// window, taping the window's substeps.  Inside the window the carried fields live in the
// tape's snapshot blocks: the window's first block is a copy of the state, and the recovery
// and diagnostics of stage i write straight into block i + 1 (after carry_block), so the
// stage start states are kept without copies; the window's end state is copied back into
// f's own fields.  Before the window the stages run on f's own fields as the step does.
int forward_taped(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields f, const StepPlan& p, const Tape& T,
                  cudaStream_t s) {
  void* stream = (void*)s;
  const bool mixed = c->precision == MPASG_PRECISION_MIXED;
  const mpasg_fields own = f;
  CHECK_RC(make_saves(m, T, f, 0, mixed, s));
  if (mixed) CHECK_RC(mpasgi_pack_f32(m, &f, s));
  CHECK_RC(mpasg_moist_coefficients(m, c, &f, stream));
  int a = 0;
  for (int sub = 1; sub <= T.hi; ++sub) {
    const bool taped = T.in(sub);
    if (sub == T.lo) {
      CHECK_RC(snap_store(m, T, f, T.snap(3 * (sub - 1)), s));
      snap_view(T, f, T.snap(3 * (sub - 1)));
    }
    for (int rk = 1; rk <= 3; ++rk) {
      const int i = (sub - 1) * 3 + rk - 1;
      const double dts = p.rk_sub[rk - 1];
      if (rk == 1 || (rk == 2 && p.order == 3)) {
        if (taped) coef_view(T, f, coef_slot(p, sub, rk));
        CHECK_RC(mpasg_vert_imp_coefs(m, c, &f, dts, stream));
      }
      CHECK_RC(mpasgi_dyn_tend(m, c, &f, rk, s, true));
      if (taped && T.n_sg > 0) CHECK_RC(mpasgi_nonneg_bytes(f.tend_u, T.sg(i), (m->nEdges + 1LL) * m->nVertLevels, s));
      CHECK_RC(mpasg_smlstep_pert(m, c, &f, stream));
      for (int small = 1; small <= p.nsub[rk - 1]; ++small) {
        if (taped) aco_redirect(T, f, a);
        CHECK_RC(mpasgi_acoustic_step(m, c, &f, small, dts, s, true));
        if (taped) CHECK_RC(aco_store(m, T, f, a, s));
        ++a;
        CHECK_RC(mpasgi_divergence_damping(m, c, &f, dts, s, true));
      }
      if (taped) {
        CHECK_RC(carry_block(m, T, T.snap(i), T.snap(i + 1), rk, s));
        snap_view(T, f, T.snap(i + 1));
      }
      CHECK_RC(mpasg_recover_large_step(m, c, &f, rk, p.nsub[rk - 1], p.rk_ts[rk - 1], stream));
      CHECK_RC(mpasgi_solve_diagnostics(m, c, &f, rk, s, true));
    }
    if (sub < p.split && sub < T.hi) CHECK_RC(make_saves(m, T, f, sub, mixed, s));
  }
  mpasg_fields out = own;
  return snap_restore(m, T, out, T.snap(3 * T.hi), s);
}

// zero every cotangent accumulator of g that is not a carried field
int zero_internal(const mpasg_mesh* m, mpasg_fields* g, cudaStream_t s) {
  const long long L = m->nVertLevels;
  const long long nel = (m->nEdges + 1LL) * L, ncw = (m->nCells + 1LL) * (L + 1), ncl = (m->nCells + 1LL) * L;
  double* e_fields[] = {g->ru_save, g->tend_u, g->tend_u_euler, g->ru_p, g->theta_edge_save};
  double* w_fields[] = {g->rw_save, g->tend_w, g->tend_w_euler, g->tend_rw, g->rw_p, g->coftz};
  double* c_fields[] = {g->rtheta_p_save, g->rho_p_save, g->theta_m_save, g->rr_save, g->tend_theta,
                        g->tend_theta_euler, g->tend_rho, g->kdiff, g->rho_pp, g->rtheta_pp, g->rtheta_pp_old,
                        g->cofwz, g->cofwt, g->a_tri, g->alpha_tri, g->gamma_tri};
  ZeroSpan zs[27];
  int n = 0;
  for (double* p : e_fields) zs[n++] = {p, nel};
  for (double* p : w_fields) zs[n++] = {p, ncw};
  for (double* p : c_fields) zs[n++] = {p, ncl};
  return mpasgi_zero_many(zs, n, s);
}

int zero_work_cotangents(const mpasg_mesh* m, mpasg_fields* g, cudaStream_t s) {
  const long long L = m->nVertLevels;
  const long long nel = (m->nEdges + 1LL) * L, ncw = (m->nCells + 1LL) * (L + 1), ncl = (m->nCells + 1LL) * L;
  const ZeroSpan zs[] = {{g->ru_p, nel}, {g->rw_p, ncw}, {g->rho_pp, ncl}, {g->rtheta_pp, ncl}, {g->rtheta_pp_old, ncl}};
  return mpasgi_zero_many(zs, 5, s);
}

// the reverse pass of one step from its tape (f supplies the static fields: base state,
// moist coefficients, diabatic forcing; its pointers are redirected into the tape)
int step_reverse(const mpasg_mesh* m, const mpasg_config* c, const mpasg_fields* fin, mpasg_fields* g,
                 const mpasg_transpose* t, const StepPlan& p, const Tape& T, const AdjWork& w, cudaStream_t s) {
  const int L = m->nVertLevels;
  const mpasg_fields f = *fin;
  // the step's last window starts from clean accumulators; a later window continues from the
  // save cotangents the previous one left (folded at the top of its first substep)
  if (T.hi == p.split) CHECK_RC(zero_internal(m, g, s));
  int a = T.hi * T.per_sub_ac;
  for (int sub = T.hi; sub >= T.lo; --sub) {
    if (sub < p.split) CHECK_RC(fold_saves(m, g, s));
    // the substep's edge mean of theta_m_save and its reciprocal sum, for the stages below
    mpasg_fields fe = f;
    sv_view(T, fe, sub - 1);
    CHECK_RC(mpasgi_theta_edge(m, &fe, false, s));
    for (int rk = 3; rk >= 1; --rk) {
      const int i = (sub - 1) * 3 + rk - 1;
      const double dts = p.rk_sub[rk - 1];
      // diagnostics and recovery: their outputs are the next RK stage's start state
      mpasg_fields post = fe;
      snap_view(T, post, T.snap(i + 1));
      CHECK_RC(mpasgi_diag_vjp_core(m, c, &post, g, t, rk, w, s));
      CHECK_RC(mpasgi_recover_vjp_core(m, c, &post, g, rk, p.rk_ts[rk - 1], w, s));
      // acoustic substeps, last first, from their taped inputs and outputs
      mpasg_fields pre = fe;
      snap_view(T, pre, T.snap(i));
      coef_view(T, pre, coef_slot(p, sub, rk));
      for (int small = p.nsub[rk - 1]; small >= 1; --small) {
        --a;
        mpasg_fields ac = pre;
        aco_view(T, ac, a);
        // the substep's inputs rtheta_pp and rw_p: the previous substep's outputs (the first
        // substep of a stage starts from zero and reads neither)
        const double* prev = T.aco(small > 1 ? a - 1 : a);
        CHECK_RC(mpasgi_divdamp_vjp_core(m, c, &ac, g, dts, w, s));
        CHECK_RC(mpasgi_acoustic_vjp_rev(m, c, &ac, g, t, small, dts, prev + T.E + 2 * T.W + T.C, prev + T.E + T.W,
                                         w, s));
      }
      CHECK_RC(mpasgi_smlstep_vjp_core(m, nullptr, T.n_sg > 0 ? T.sg(i) : nullptr, g, s));
      CHECK_RC(mpasgi_dyn_tend_vjp_core(m, c, &pre, g, t, rk, w, s));
      if (rk == 1 || (rk == 2 && p.order == 3)) CHECK_RC(mpasgi_vimp_vjp_core(m, c, &pre, g, dts, w, s));
      // every RK stage starts its acoustic perturbations from zero
      CHECK_RC(zero_work_cotangents(m, g, s));
    }
    // the edge-sum cotangent of this substep's theta_m_save, gathered on the cells
    k_theta_edge_vjp<<<nblocks((long long)m->nCells * L), kBlock, 0, s>>>(*m, *g, FastDiv(L));
    MPASG_LAUNCH_CHECK();
    CHECK_RC(mpasgi_zero(g->theta_edge_save, (m->nEdges + 1LL) * L, s));
  }
  return T.lo == 1 ? fold_saves(m, g, s) : MPASG_OK;
}

// the reverse pass is float64 in both forms: the mixed form's gradient is the float64
// linearisation about the mixed trajectory
bool step_args_ok(const mpasg_mesh* m, const mpasg_config* c) {
  return adj_supported(m, c) && (c->precision == MPASG_PRECISION_FLOAT64 || c->precision == MPASG_PRECISION_MIXED) &&
         (c->time_integration_order == 2 || c->time_integration_order == 3) && c->number_of_sub_steps >= 1 &&
         c->dynamics_split_steps >= 1;
}

}  // namespace

extern "C" long long mpasg_step_vjp_tape_doubles(const mpasg_mesh* m, const mpasg_config* c) {
  if (!m || !c || c->dynamics_split_steps < 1 || c->number_of_sub_steps < 1) return -1;
  const StepPlan p = plan_of(c);
  return Tape(m, p).doubles();
}

extern "C" int mpasg_step_tape(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, double* tape,
                               void* stream) {
  if (!m || !c || !f || !tape || !step_args_ok(m, c)) return MPASG_E_ARG;
  const StepPlan p = plan_of(c);
  Tape T(m, p);
  T.base = tape;
  return forward_taped(m, c, *f, p, T, (cudaStream_t)stream);
}

extern "C" int mpasg_step_vjp_taped(const mpasg_mesh* m, const mpasg_config* c, const mpasg_fields* f,
                                    mpasg_fields* g, const mpasg_transpose* t, const double* tape, double* work,
                                    void* stream) {
  if (!m || !c || !f || !g || !t || !tape || !work || !step_args_ok(m, c)) return MPASG_E_ARG;
  const StepPlan p = plan_of(c);
  Tape T(m, p);
  T.base = const_cast<double*>(tape);  // read only below
  return step_reverse(m, c, f, g, t, p, T, adj_work(m, work), (cudaStream_t)stream);
}

extern "C" int mpasg_step_vjp(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, mpasg_fields* g,
                              const mpasg_transpose* t, double* tape, double* work, void* stream) {
  if (!m || !c || !f || !g || !t || !tape || !work || !step_args_ok(m, c)) return MPASG_E_ARG;
  const int rc = mpasg_step_tape(m, c, f, tape, stream);
  if (rc != MPASG_OK) return rc;
  return mpasg_step_vjp_taped(m, c, f, g, t, tape, work, stream);
}

extern "C" long long mpasg_step_vjp_window_tape_doubles(const mpasg_mesh* m, const mpasg_config* c, int nsub) {
  if (!m || !c || c->dynamics_split_steps < 1 || c->number_of_sub_steps < 1 || nsub < 1 ||
      nsub > c->dynamics_split_steps)
    return -1;
  const StepPlan p = plan_of(c);
  return Tape(m, p, 1, nsub).doubles();
}

extern "C" int mpasg_step_vjp_window(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, mpasg_fields* g,
                                     const mpasg_transpose* t, double* tape, double* work, int sub_lo, int sub_hi,
                                     void* stream) {
  if (!m || !c || !f || !g || !t || !tape || !work || !step_args_ok(m, c)) return MPASG_E_ARG;
  if (sub_lo < 1 || sub_hi < sub_lo || sub_hi > c->dynamics_split_steps) return MPASG_E_ARG;
  const StepPlan p = plan_of(c);
  Tape T(m, p, sub_lo, sub_hi);
  T.base = tape;
  cudaStream_t s = (cudaStream_t)stream;
  const int rc = forward_taped(m, c, *f, p, T, s);
  if (rc != MPASG_OK) return rc;
  return step_reverse(m, c, f, g, t, p, T, adj_work(m, work), s);
}
