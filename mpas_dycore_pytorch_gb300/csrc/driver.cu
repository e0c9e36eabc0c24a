// Native large-step driver (the reference's atm_srk3, mpas_pytorch/dynamics/time_integration.py:
// 4897 / :3420): RK integration setup (:2497), 3 dynamics substeps x 3 RK stages
// (execute_rk_step :5000), split-transport bookkeeping (:3825-3942), the split transport RK3
// loop (:3954-4700) and the final reconstruction (:4729).  All work is enqueued on the
// caller's stream without host synchronisation, so the whole step can be captured in a
// CUDA graph by the caller.
#include <cmath>
#include <cstdio>

#include "common.cuh"

namespace {

__global__ void k_fill_d(double* __restrict__ p, long long n, double v) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

__global__ void k_add_d(double* __restrict__ y, const double* __restrict__ x, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = y[i] + x[i];
}

__global__ void k_scale_d(double* __restrict__ y, const double* __restrict__ x, double a, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = x[i] * a;
}

__global__ void k_count_nonfinite(const double* __restrict__ p, long long n, int32_t* __restrict__ count) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int bad = 0;
  if (i < n) bad = isfinite(p[i]) ? 0 : 1;
  bad = __syncthreads_count(bad);
  if (threadIdx.x == 0 && bad) atomicAdd(count, bad);
}

// mixed-form arithmetic helpers applied elementwise (mpasg_numerics_check)
__global__ void k_numerics(int which, const double* __restrict__ in, double* __restrict__ out, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double x = in[i];
  out[i] = which == 0 ? f2d_bits(d2f_bits(x)) : rcp_nr(x);
}

// float32 copies of float64 fields (mixed form), one launch for up to four arrays
struct PackJob {
  const double* src[4];
  float* dst[4];
  long long n[4];
};

__global__ void k_pack_f32(PackJob job) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int a = blockIdx.y;
  // select with constant indices (a dynamic index into the parameter struct would copy
  // it to local memory in every thread)
  const double* src = a == 0 ? job.src[0] : a == 1 ? job.src[1] : a == 2 ? job.src[2] : job.src[3];
  float* dst = a == 0 ? job.dst[0] : a == 1 ? job.dst[1] : a == 2 ? job.dst[2] : job.dst[3];
  const long long n = a == 0 ? job.n[0] : a == 1 ? job.n[1] : a == 2 ? job.n[2] : job.n[3];
  if (i < n) dst[i] = d2f_bits(src[i]);
}

// dst row i = src row rows[i] (rows of row_len float64 values)
__global__ void k_permute_rows(const double* __restrict__ src, double* __restrict__ dst,
                               const long long* __restrict__ rows, long long n, long long row_len) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * row_len) return;
  const long long r = i / row_len, j = i - r * row_len;
  dst[i] = src[rows[r] * row_len + j];
}

int fill(double* p, long long n, double v, cudaStream_t s) {
  k_fill_d<<<nblocks(n), kBlock, 0, s>>>(p, n, v);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

int copy(double* dst, const double* src, long long n, cudaStream_t s) {
  if (cudaMemcpyAsync(dst, src, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return MPASG_E_CUDA;
  return MPASG_OK;
}

#define CHECK_RC(x)          \
  do {                       \
    int _rc = (x);           \
    if (_rc != MPASG_OK) return _rc; \
  } while (0)

}  // namespace

static long long g_launches = 0;
void mpasg_count_launch() { __atomic_add_fetch(&g_launches, 1, __ATOMIC_RELAXED); }
extern "C" long long mpasg_launch_count(void) { return __atomic_load_n(&g_launches, __ATOMIC_RELAXED); }

extern "C" int mpasg_abi_version(void) { return MPASG_ABI_VERSION; }

extern "C" const char* mpasg_build_info(void) {
  static char buf[160];
  snprintf(buf, sizeof(buf), "mpasg abi=%d cuda=%d arch=sm_103a float64+mixed", MPASG_ABI_VERSION, CUDART_VERSION);
  return buf;
}

int mpasgi_pack_f32(const mpasg_mesh* m, mpasg_fields* f, cudaStream_t s) {
  const long long L = m->nVertLevels;
  const long long nel = (m->nEdges + 1) * L, ncw = (m->nCells + 1) * (L + 1);
  PackJob job{{f->u, f->pv_edge, f->w, f->rw}, {f->u_f32, f->pv_edge_f32, f->w_f32, f->rw_f32}, {nel, nel, ncw, ncw}};
  for (int a = 0; a < 4; ++a)
    if (!job.src[a] || !job.dst[a]) return MPASG_E_ARG;
  dim3 grid(nblocks(nel > ncw ? nel : ncw), 4);
  k_pack_f32<<<grid, kBlock, 0, s>>>(job);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

extern "C" int mpasg_permute_rows(const double* src, double* dst, const long long* rows, long long n,
                                  long long row_len, void* stream) {
  if (!src || !dst || !rows || n < 0 || row_len < 1 || src == dst) return MPASG_E_ARG;
  if (n == 0) return MPASG_OK;
  k_permute_rows<<<nblocks(n * row_len), kBlock, 0, (cudaStream_t)stream>>>(src, dst, rows, n, row_len);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

extern "C" int mpasg_numerics_check(int which, const double* in, double* out, long long n, void* stream) {
  if (!in || !out || n < 0 || (which != 0 && which != 1)) return MPASG_E_ARG;
  if (n == 0) return MPASG_OK;
  k_numerics<<<nblocks(n), kBlock, 0, (cudaStream_t)stream>>>(which, in, out, n);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

namespace {
// 8 independent multiply-add chains per thread: the float64 pipe, not latency, bounds it
__global__ void __launch_bounds__(256) k_fp64_peak(double* buf, int iters) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const double x = buf[t], y = 1.0 - x;
  double a[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) a[j] = x + (double)j;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = fma(a[j], x, y);
  }
  double sum = 0.0;
#pragma unroll
  for (int j = 0; j < 8; ++j) sum += a[j];
  buf[t] = sum;
}
}  // namespace

extern "C" int mpasg_fp64_peak(double* buf, int blocks, int iters, double* flops_per_s, void* stream) {
  if (!buf || !flops_per_s || blocks < 1 || iters < 1) return MPASG_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  cudaEvent_t a, b;
  if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) return MPASG_E_CUDA;
  int rc = MPASG_OK;
  float ms = 0.0f;
  for (int rep = 0; rep < 2 && rc == MPASG_OK; ++rep) {
    if (rep == 1 && cudaEventRecord(a, s) != cudaSuccess) rc = MPASG_E_CUDA;
    k_fp64_peak<<<blocks, 256, 0, s>>>(buf, iters);
    mpasg_count_launch();
    if (cudaGetLastError() != cudaSuccess) rc = MPASG_E_LAUNCH;
  }
  if (rc == MPASG_OK && (cudaEventRecord(b, s) != cudaSuccess || cudaEventSynchronize(b) != cudaSuccess ||
                         cudaEventElapsedTime(&ms, a, b) != cudaSuccess))
    rc = MPASG_E_CUDA;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc == MPASG_OK) *flops_per_s = 2.0 * 8.0 * (double)iters * (double)blocks * 256.0 / ((double)ms * 1e-3);
  return rc;
}

extern "C" int mpasg_check_finite(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, void* stream) {
  if (!m || !c || !f || !f->status) return MPASG_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const long long L = m->nVertLevels, nc = m->nCells, ne = m->nEdges;
  if (cudaMemsetAsync(f->status, 0, sizeof(int32_t), s) != cudaSuccess) return MPASG_E_CUDA;
  struct Item { const double* p; long long n; } items[] = {
      {f->u, ne * L}, {f->w, nc * (L + 1)}, {f->theta_m, nc * L}, {f->rho_zz, nc * L},
      {f->scalars, nc * L * c->num_scalars}};
  for (auto& it : items) {
    if (it.n <= 0) continue;
    k_count_nonfinite<<<nblocks(it.n), kBlock, 0, s>>>(it.p, it.n, f->status);
    MPASG_LAUNCH_CHECK();
  }
  return MPASG_OK;
}

namespace {
// Records one CUDA event at every stage boundary of the step (stage kinds in `kinds`).
struct StageRecorder {
  cudaEvent_t* events = nullptr;
  int n_events = 0;
  int32_t* kinds = nullptr;
  int n = 0;
  int mark(int kind, cudaStream_t s) {
    if (kinds && n < n_events) kinds[n] = kind;
    if (events && n < n_events) {
      cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
      cudaStreamIsCapturing(s, &st);
      cudaError_t e = (st == cudaStreamCaptureStatusActive)
                          ? cudaEventRecordWithFlags(events[n], s, cudaEventRecordExternal)
                          : cudaEventRecord(events[n], s);
      if (e != cudaSuccess) return MPASG_E_CUDA;
    }
    ++n;
    return MPASG_OK;
  }
};

int step_impl(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* fin, cudaStream_t s, StageRecorder* rec,
              double* tape = nullptr, int part = -1);
}  // namespace

extern "C" int mpasg_step(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* fin, void* stream) {
  if (!m || !c || !fin) return MPASG_E_ARG;
  return step_impl(m, c, fin, (cudaStream_t)stream, nullptr);
}

extern "C" int mpasg_step_part(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* fin, int part,
                               void* stream) {
  if (!m || !c || !fin || (part != 0 && part != 1)) return MPASG_E_ARG;
  return step_impl(m, c, fin, (cudaStream_t)stream, nullptr, nullptr, part);
}

extern "C" int mpasg_step_taped(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* fin, double* tape,
                                void* stream) {
  if (!m || !c || !fin || !tape || c->dynamics_split_steps != 1 || c->num_scalars < 1) return MPASG_E_ARG;
  return step_impl(m, c, fin, (cudaStream_t)stream, nullptr, tape);
}

extern "C" int mpasg_step_timed(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* fin, void* const* events,
                                int32_t* stage_kinds, int n_events, void* stream) {
  if (!m || !c || !fin || n_events < 0) return MPASG_E_ARG;
  StageRecorder rec;
  rec.events = (cudaEvent_t*)events;
  rec.kinds = stage_kinds;
  rec.n_events = n_events;
  int rc = step_impl(m, c, fin, (cudaStream_t)stream, &rec);
  if (rc != MPASG_OK) return rc;
  return rec.n;  // number of boundaries recorded (>= 0)
}

namespace {
// One transport RK stage, scalars_init and scalars_a -> scalars_b, then a and b swap:
// monotone at the last stage when config_monotonic, else explicit.
int transport_stage(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, int rk, double dt_stage,
                    cudaStream_t s) {
  const int rc = (rk == 3 && c->monotonic) ? mpasg_advance_scalars_mono(m, c, f, dt_stage, (void*)s)
                                           : mpasg_advance_scalars(m, c, f, rk, dt_stage, (void*)s);
  if (rc != MPASG_OK) return rc;
  double* t = f->scalars_a;
  f->scalars_a = f->scalars_b;
  f->scalars_b = t;
  return MPASG_OK;
}

#define MARK(kind)                                  \
  do {                                              \
    if (rec) CHECK_RC(rec->mark((kind), s));        \
  } while (0)

// The end of a large step: the split transport RK3 with the substep-averaged mass fluxes
// (the coupled mode advanced the scalars inside the RK stages already) and the final
// scalars.  Of the step boundary it writes only the scalars.
int step_tail(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields f, cudaStream_t s, StageRecorder* rec) {
  const long long L = m->nVertLevels, nc = m->nCells;
  const long long S = c->num_scalars;
  const bool advect = S > 0 && !c->scalar_advection_off;
  const bool coupled = c->dynamics_split_steps == 1;
  const double dt = c->dt;
  if (advect && !coupled) {
    CHECK_RC(copy(f.scalars_a, f.scalars_init, (nc + 1) * L * S, s));
    // transport stage dts; the first is dt/2 for RK2 (time_integration.py:3366-3370)
    const double dts_t[3] = {c->time_integration_order == 2 ? dt / 2.0 : dt / 3.0, dt / 2.0, dt};
    MARK(MPASG_STAGE_SPLIT);
    for (int rk = 1; rk <= 3; ++rk) {
      CHECK_RC(transport_stage(m, c, &f, rk, dts_t[rk - 1], s));
      MARK(rk == 3 && c->monotonic ? MPASG_STAGE_SCALARS_MONO : MPASG_STAGE_SCALARS);
    }
    // active rows only: the padding row of the scalars passes through the step unchanged,
    // as in the reference
    CHECK_RC(copy(f.scalars, f.scalars_a, nc * L * S, s));
    MARK(MPASG_STAGE_SPLIT);
  }
  return MPASG_OK;
}

// part -1: the whole step; 0: everything but the split transport (every field of the
// step boundary but the scalars is final after it; the reconstruction reads u only, so
// it runs before the transport); 1: step_tail
int step_impl(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* fin, cudaStream_t s, StageRecorder* rec,
              double* tape, int part) {
  void* stream = (void*)s;
  if (c->time_integration_order != 2 && c->time_integration_order != 3) return MPASG_E_ARG;
  if (c->number_of_sub_steps < 1 || c->dynamics_split_steps < 1) return MPASG_E_ARG;
  mpasg_fields f = *fin;  // local copy: transport ping-pongs its scalar buffers
  if (part == 1) return step_tail(m, c, f, s, rec);
  const long long L = m->nVertLevels, nc = m->nCells, ne = m->nEdges;
  const long long S = c->num_scalars;
  const bool advect = S > 0 && !c->scalar_advection_off;  // config_scalar_advection
  const long long ncl = (nc + 1) * L, nel = (ne + 1) * L, ncw = (nc + 1) * (L + 1);
  const long long ncs = (nc + 1) * L * S;
  const int split = c->dynamics_split_steps;
  // one dynamics substep is the coupled mode: the scalars advance inside every RK stage
  // (after recovery, before the diagnostics), not in a transport loop after the substeps
  const bool coupled = split == 1;
  const int ns = c->number_of_sub_steps;
  const double dt = c->dt;
  const double dt_dyn = dt / split;
  double rk_ts[3], rk_sub[3];
  int nsub[3];
  if (c->time_integration_order == 3) {
    rk_ts[0] = dt_dyn / 3.0; rk_ts[1] = dt_dyn / 2.0; rk_ts[2] = dt_dyn;
    rk_sub[0] = dt_dyn / 3.0; rk_sub[1] = dt_dyn / ns; rk_sub[2] = dt_dyn / ns;
    nsub[0] = 1; nsub[1] = ns / 2 > 1 ? ns / 2 : 1; nsub[2] = ns;
  } else {
    rk_ts[0] = dt_dyn / 2.0; rk_ts[1] = dt_dyn / 2.0; rk_ts[2] = dt_dyn;
    rk_sub[0] = rk_sub[1] = rk_sub[2] = dt_dyn / ns;
    nsub[0] = nsub[1] = ns / 2 > 1 ? ns / 2 : 1; nsub[2] = ns;
  }

  // ---- RK integration setup
  MARK(MPASG_STAGE_BEGIN);
  CHECK_RC(fill(f.theta_m + nc * L, L, 0.0, s));
  CHECK_RC(copy(f.ru_save, f.ru, nel, s));
  CHECK_RC(copy(f.rw_save, f.rw, ncw, s));
  CHECK_RC(copy(f.rtheta_p_save, f.rtheta_p, ncl, s));
  CHECK_RC(copy(f.rho_p_save, f.rho_p, ncl, s));
  CHECK_RC(copy(f.theta_m_save, f.theta_m, ncl, s));
  CHECK_RC(copy(f.rr_save, f.rho_p, ncl, s));
  CHECK_RC(copy(f.rho_zz_old_split, f.rho_zz, ncl, s));
  if (S > 0) CHECK_RC(copy(f.scalars_init, f.scalars, ncs, s));
  if (advect && coupled) CHECK_RC(copy(f.scalars_a, f.scalars_init, ncs, s));
  if (c->precision == MPASG_PRECISION_MIXED) CHECK_RC(mpasgi_pack_f32(m, &f, s));
  // edge mean of theta_m_save and its reciprocal sum
  CHECK_RC(mpasgi_theta_edge(m, &f, c->precision == MPASG_PRECISION_MIXED, s));
  MARK(MPASG_STAGE_SETUP);
  CHECK_RC(mpasg_moist_coefficients(m, c, &f, stream));
  MARK(MPASG_STAGE_MOIST);

  for (int sub = 1; sub <= split; ++sub) {
    for (int rk = 1; rk <= 3; ++rk) {
      const double dts = rk_sub[rk - 1];
      if (rk == 1 || (rk == 2 && c->time_integration_order == 3))
      {
        CHECK_RC(mpasg_vert_imp_coefs(m, c, &f, dts, stream));
        MARK(MPASG_STAGE_VIMP);
      }
      CHECK_RC(mpasgi_dyn_tend(m, c, &f, rk, s, true));
      MARK(rk == 1 ? MPASG_STAGE_DYN_TEND_RK1 : MPASG_STAGE_DYN_TEND);
      CHECK_RC(mpasg_smlstep_pert(m, c, &f, stream));
      MARK(MPASG_STAGE_SMLSTEP);
      for (int small = 1; small <= nsub[rk - 1]; ++small) {
        CHECK_RC(mpasgi_acoustic_step(m, c, &f, small, dts, s, true));
        MARK(MPASG_STAGE_ACOUSTIC);
        CHECK_RC(mpasgi_divergence_damping(m, c, &f, dts, s, true));
        MARK(MPASG_STAGE_DIVDAMP);
      }
      CHECK_RC(mpasg_recover_large_step(m, c, &f, rk, nsub[rk - 1], rk_ts[rk - 1], stream));
      MARK(MPASG_STAGE_RECOVER);
      if (coupled && advect) {  // time_integration.py:7890-8200: stage dt, this stage's mass fluxes
        CHECK_RC(transport_stage(m, c, &f, rk, rk_ts[rk - 1], s));
        MARK(rk == 3 && c->monotonic ? MPASG_STAGE_SCALARS_MONO : MPASG_STAGE_SCALARS);
        if (tape) {  // the stage's transport inputs, for the scalar derivatives
          double* t = tape + (rk - 1) * (nel + ncw + ncl);
          CHECK_RC(copy(t, f.ruAvg, nel, s));
          CHECK_RC(copy(t + nel, f.wwAvg, ncw, s));
          CHECK_RC(copy(t + nel + ncw, f.rho_zz, ncl, s));
        }
      }
      CHECK_RC(mpasgi_solve_diagnostics(m, c, &f, rk, s, true));
      MARK(MPASG_STAGE_DIAG);
    }
    // split bookkeeping
    if (sub == 1) {
      CHECK_RC(copy(f.ruAvg_split, f.ruAvg, nel, s));
      CHECK_RC(copy(f.wwAvg_split, f.wwAvg, ncw, s));
    } else {
      k_add_d<<<nblocks(nel), kBlock, 0, s>>>(f.ruAvg_split, f.ruAvg, nel);
      MPASG_LAUNCH_CHECK();
      k_add_d<<<nblocks(ncw), kBlock, 0, s>>>(f.wwAvg_split, f.wwAvg, ncw);
      MPASG_LAUNCH_CHECK();
    }
    if (sub < split) {
      CHECK_RC(fill(f.theta_m + nc * L, L, 0.0, s));
      CHECK_RC(copy(f.ru_save, f.ru, nel, s));
      CHECK_RC(copy(f.rw_save, f.rw, ncw, s));
      CHECK_RC(copy(f.rtheta_p_save, f.rtheta_p, ncl, s));
      CHECK_RC(copy(f.rho_p_save, f.rho_p, ncl, s));
      CHECK_RC(copy(f.theta_m_save, f.theta_m, ncl, s));
      CHECK_RC(copy(f.rr_save, f.rho_p, ncl, s));
      CHECK_RC(mpasgi_theta_edge(m, &f, c->precision == MPASG_PRECISION_MIXED, s));
    }
  }
  MARK(MPASG_STAGE_SPLIT);
  const double inv = 1.0 / (double)split;
  k_scale_d<<<nblocks(nel), kBlock, 0, s>>>(f.ruAvg, f.ruAvg_split, inv, nel);
  MPASG_LAUNCH_CHECK();
  k_scale_d<<<nblocks(ncw), kBlock, 0, s>>>(f.wwAvg, f.wwAvg_split, inv, ncw);
  MPASG_LAUNCH_CHECK();
  // coupled mode: the scalars of the last RK stage are the step's (active rows only)
  if (advect && coupled) CHECK_RC(copy(f.scalars, f.scalars_a, nc * L * S, s));
  MARK(MPASG_STAGE_SPLIT);
  CHECK_RC(mpasgi_reconstruct(m, c, &f, s, true));
  MARK(MPASG_STAGE_RECONSTRUCT);
  if (part == 0) return MPASG_OK;
  return step_tail(m, c, *fin, s, rec);
}
#undef MARK
}  // namespace
