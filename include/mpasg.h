/*
 * mpasg.h -- C ABI of the GB300 (sm_103a) implementation of the MPAS split-explicit
 * dynamics timestep (the reference's atm_srk3 hot path).
 *
 * Every entry point takes plain POD structs of DEVICE pointers plus a cudaStream_t
 * (passed as void*), launches asynchronously on that stream and returns an int status
 * (MPASG_OK or a negative MPASG_E_* code). No entry point allocates device memory:
 * callers own every buffer (the Python host allocates them from one arena), except the
 * fixed edge scratch compiled into the library for mpasg_advance_scalars_static.
 *
 * Layout (matches the reference's runtime tensors, so host<->device needs no transpose):
 *   cell / edge / vertex fields are row-major (N+1, L) float64, levels fastest, with one
 *   trailing padding row; W-level fields are (N+1, L+1); scalars are (C+1, L, S).
 *   Connectivity is 0-based int32; a missing neighbour points at the padding row
 *   (index N), which holds zeros (rho_zz holds 1.0 there, as in the reference).
 *
 * Reference interfaces replaced (NOAA-EMC/mpas-dycore-pytorch v0.1.7, mpas_pytorch/):
 *   mpasg_step                  dynamics/time_integration.py:4897  atm_srk3 (+ :3420 _atm_srk3_impl)
 *   mpasg_prepare               atmosphere_model.py:782  _prepare_timestep_state
 *                               (dynamics/init_coupled_diagnostics.py:147)
 *   mpasg_prepare_derived       the same from theta_m / rho_zz (init_coupled_diagnostics.py:259)
 *   mpasg_digest                state.py:72,85 (value binding of a complete step boundary)
 *   mpasg_moist_coefficients    dynamics/moist_coefficients.py:124
 *   mpasg_vert_imp_coefs        dynamics/vert_imp_coefs.py:188
 *   mpasg_dyn_tend              dynamics/dyn_tend.py:10836  atm_compute_dyn_tend_work
 *   mpasg_smlstep_pert          dynamics/smlstep_pert.py:373
 *   mpasg_acoustic_step         dynamics/acoustic_step.py:1297
 *   mpasg_divergence_damping    dynamics/divergence_damping.py:299
 *   mpasg_recover_large_step    dynamics/recover_large_step.py:1090
 *   mpasg_solve_diagnostics     dynamics/solve_diagnostics.py:1052
 *   mpasg_advance_scalars       dynamics/advance_scalars.py:1272
 *   mpasg_advance_scalars_mono  dynamics/advance_scalars_mono.py:2878
 *   mpasg_reconstruct_2d        dynamics/vector_reconstruction.py:311
 *   mpasg_surface_pressure      diagnostics.py:10  physics_interface_surface_pressure
 *   mpasg_surface_pressure_vjp / _jvp, mpasg_weighted_sq_sum_vjp
 *                               torch autograd through diagnostics.py:77-82 (reverse / forward mode)
 *   mpasg_sfc_order, mpasg_edge_order  mesh_reordering.py:106 compute_rcm_permutation (SFC orders)
 *   mpasg_tridiag_*             autodiff/tridiagonal_solve.py:177, autodiff/tridiagonal_factor.py:145
 *   mpasg_advance_scalars_static  (no counterpart: advance_scalars.py:1272 without caller scratch)
 *   mpasg_step_vjp, mpasg_prepare_vjp, mpasg_*_vjp (dynamics stages)
 *                               torch autograd through atmosphere_model.py:2101 _run_simulation_vjp /
 *                               dynamics/time_integration.py:4897 atm_srk3(differentiable=True)
 *   mpasg_step_jvp, mpasg_prepare_jvp, mpasg_*_jvp (dynamics stages)
 *                               torch forward-mode AD through atmosphere_model.py:2041 _run_simulation_jvp
 */
#ifndef MPASG_H
#define MPASG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MPASG_ABI_VERSION 4

enum {
  MPASG_OK = 0,
  MPASG_E_ARG = -1,      /* null pointer / bad dimension / unsupported option */
  MPASG_E_LAUNCH = -2,   /* a kernel launch failed (cudaGetLastError) */
  MPASG_E_NONFINITE = -3,/* the finite-field check found NaN/Inf */
  MPASG_E_CUDA = -4,     /* another CUDA runtime error */
  MPASG_E_SCRATCH = -5   /* the problem exceeds the library-owned static scratch */
};

/* Static mesh: dimensions, connectivity, geometry and vertical metrics. */
typedef struct mpasg_mesh {
  int32_t nCells, nEdges, nVertices, nVertLevels;
  int32_t maxEdges, maxEdges2, vertexDegree, nAdvMax;
  int32_t flatTerrain;   /* 1 when zb_cell == zb3_cell == zxu == 0: terrain-slope terms are skipped */
  int32_t reserved0;
  double cf1, cf2, cf3;
  /* connectivity (0-based; missing -> padding row) */
  const int32_t *nEdgesOnCell;      /* (C)            */
  const int32_t *edgesOnCell;       /* (C, maxEdges)  */
  const int32_t *cellsOnCell;       /* (C, maxEdges)  */
  const int32_t *verticesOnCell;    /* (C, maxEdges)  */
  const int32_t *kiteForCell;       /* (C, maxEdges) 0-based slot in cellsOnVertex, -1 if none */
  const int32_t *cellsOnEdge;       /* (E, 2)         */
  const int32_t *verticesOnEdge;    /* (E, 2)         */
  const int32_t *nEdgesOnEdge;      /* (E)            */
  const int32_t *edgesOnEdge;       /* (E, maxEdges2) */
  const int32_t *nAdvCellsForEdge;  /* (E)            */
  const int32_t *advCellsForEdge;   /* (E, nAdvMax)   */
  const int32_t *edgesOnVertex;     /* (V, vertexDegree) */
  /* geometry (float64) */
  const double *edgesOnCell_sign;   /* (C, maxEdges) */
  const double *edgesOnVertex_sign; /* (V, vertexDegree) */
  const double *dcEdge, *dvEdge, *invDcEdge, *invDvEdge;       /* (E+1) */
  const double *invAreaCell;        /* (C+1) */
  const double *invAreaTriangle;    /* (V+1) */
  const double *kiteAreasOnVertex;  /* (V, vertexDegree) */
  const double *weightsOnEdge;      /* (E, maxEdges2) */
  const double *adv_coefs, *adv_coefs_3rd;   /* (E, nAdvMax) */
  const double *adv_coefs_p, *adv_coefs_m;   /* (E, nAdvMax): adv_coefs +/- adv_coefs_3rd */
  const double *defc_a, *defc_b;    /* (C, maxEdges) */
  const double *fEdge;              /* (E+1) */
  const double *fVertex;            /* (V+1) */
  const double *meshScalingDel2, *meshScalingDel4;  /* (E+1) */
  const double *latCell, *lonCell;  /* (C+1) */
  const double *coeffs_reconstruct; /* (C, maxEdges, 3) */
  const double *zb_cell, *zb3_cell; /* (C, maxEdges, L+1) */
  const double *zxu;                /* (E+1, L) */
  const double *zz;                 /* (C+1, L) */
  const double *dss;                /* (C+1, L) */
  const double *rho_base, *theta_base;  /* (C+1, L) */
  const double *rdzw, *rdzu, *fzm, *fzp, *fnm, *fnp, *rdnw;    /* (L) */
  /* Reference theta profile of the mixed form (float64): ref_theta (L) is the base-state
   * theta of the first cell; at each w interface k (L+1 values, zero where unused) its vertical
   * flux weights: ref_theta_w4 / ref_theta_w3 are the centred and upwind parts of the
   * third-order interpolation (2 <= k <= L-2), ref_theta_w2 = fzm ref_k + fzp ref_(k-1)
   * (1 <= k <= L-1). */
  const double *ref_theta, *ref_theta_w4, *ref_theta_w3, *ref_theta_w2;
  /* float32 copies of the geometry the mixed form's stencils read (same shapes as above) */
  const float *edgesOnCell_sign_f32, *edgesOnVertex_sign_f32, *dcEdge_f32, *dvEdge_f32,
      *invDcEdge_f32, *invDvEdge_f32, *invAreaCell_f32, *invAreaTriangle_f32,
      *kiteAreasOnVertex_f32, *weightsOnEdge_f32, *adv_coefs_p_f32, *adv_coefs_m_f32,
      *defc_a_f32, *defc_b_f32, *meshScalingDel2_f32, *meshScalingDel4_f32,
      *coeffs_reconstruct_f32, *zxu_f32, *zz_f32, *rdzw_f32, *rdzu_f32, *fzm_f32, *fzp_f32,
      *fnm_f32, *fnp_f32, *rdnw_f32;
  /* interface heights (C+1, L+1): the vertical mixing options of the tendencies */
  const double *zgrid;
  /* initial profiles read by config_mix_full = false: u_init, v_init (L), angleEdge (E+1),
   * t_init (C+1, L) */
  const double *u_init, *v_init, *angleEdge, *t_init;
  /* (C+1, maxEdges): edgesOnCell_sign * dvEdge * invAreaCell of every cell's edge slots
   * (the divergence weight of the acoustic flux sums) */
  const double *cell_edge_geo;
  /* (C+1, maxEdges) products the stencils would otherwise form at every level, each in the
   * association the kernels use: edgesOnCell_sign * dvEdge; the del2 mixing weights
   * 0.5 * invAreaCell * sign * dvEdge * invDcEdge (w) and invAreaCell * sign * dvEdge *
   * invDcEdge (theta) */
  const double *cell_edge_sdv, *cell_edge_es_w, *cell_edge_es_t;
  /* dcEdge * dvEdge (E+1) and edgesOnVertex_sign * dcEdge (V+1, vertexDegree), formed once */
  const double *edge_dcdv, *vertex_edge_sdc;
  /* (C+1, 4): cos latCell, sin latCell, cos lonCell, sin lonCell (reconstruction) */
  const double *cell_trig;
} mpasg_mesh;

/* Namelist options the step consumes (validated on the host). */
typedef struct mpasg_config {
  double dt;                 /* large timestep (s) */
  double epssm, smdiv, len_disp, coef_3rd_order, c_s;
  double visc4_2dsmag, del4u_div_factor, apvm_upwinding;
  double h_mom_eddy_visc4, h_theta_eddy_visc4;  /* used when horiz_mixing != 2d_smagorinsky */
  int32_t time_integration_order;   /* 2 or 3 */
  int32_t number_of_sub_steps;      /* acoustic substeps ns */
  int32_t dynamics_split_steps;     /* split */
  int32_t monotonic;                /* monotone limiter on the last transport stage */
  int32_t horiz_mixing_smagorinsky; /* 1: 2d_smagorinsky */
  int32_t num_scalars, moist_start, moist_end;
  int32_t precision;                /* MPASG_PRECISION_FLOAT64 or MPASG_PRECISION_MIXED */
  int32_t tile_tend_u;              /* levels per thread of the u tendency: 1 (0), 2 or 4
                                       (autotuned; tiles agree to one FMA rounding) */
  /* mixing options of the large-step tendencies (dyn_tend.py:3367-3456, 2730-2780,
   * 4612-4650, 5064-5100): 2d_fixed del2 coefficient (kdiff everywhere), vertical mixing
   * of u and w / of theta (full state; 0 = off), CAM-style top-level damping (0 = off) */
  double h_theta_eddy_visc2, v_mom_eddy_visc2, v_theta_eddy_visc2, mpas_cam_coef;
  int32_t number_cam_damping_levels;
  int32_t scalar_advection_off;     /* 1: config_scalar_advection = false (scalars not transported) */
  /* Rayleigh damping of u on the top levels (every RK stage; dyn_tend.py:10066-10072,
   * 2956-2990) and vertical mixing of the perturbation from the initial profiles */
  double rayleigh_damp_u_timescale_days;
  int32_t rayleigh_damp_u_levels;   /* 0: off */
  int32_t mix_perturbation;         /* 1: config_mix_full = false */
} mpasg_config;

/* Arithmetic of the step.  FLOAT64: every stage in float64 (the reference's arithmetic).
 * MIXED: fields stay float64 in memory and the float64 parts below stay float64; the
 * horizontal stencils (tendencies, fluxes, transport, diagnostics, damping) evaluate
 * in float32.  Float64 parts: vertically implicit coefficients and the tridiagonal
 * solve, recovery of the prognostic state including Exner function and pressure
 * perturbation, accumulation of the acoustic perturbations and of the RK stages. */
enum { MPASG_PRECISION_FLOAT64 = 0, MPASG_PRECISION_MIXED = 1 };

/*
 * Every device array the step touches: the carried state (reference key names), the
 * per-step work arrays, and scratch. All pointers are device pointers; shapes use
 * C, E, V, L, S (cells, edges, vertices, levels, scalars), each with a padding row.
 */
typedef struct mpasg_fields {
  /* carried state / diagnostics */
  double *u, *v, *ru, *ruAvg, *h_edge, *pv_edge;                    /* (E+1, L) */
  double *w, *rw, *wwAvg;                                           /* (C+1, L+1) */
  double *theta_m, *rho_zz, *rho_p, *rtheta_p, *rtheta_base, *exner, *exner_base,
         *pressure_p, *pressure_base, *divergence, *ke, *rt_diabatic_tend;  /* (C+1, L) */
  double *uReconstructX, *uReconstructY, *uReconstructZ,
         *uReconstructZonal, *uReconstructMeridional;               /* (C+1, L) */
  double *vorticity;                                                /* (V+1, L) */
  double *scalars;                                                  /* (C+1, L, S) */
  /* RK-step saves and split bookkeeping */
  double *ru_save, *ruAvg_split;                                    /* (E+1, L) */
  double *rw_save, *wwAvg_split;                                    /* (C+1, L+1) */
  double *rtheta_p_save, *rho_p_save, *theta_m_save, *rr_save, *rho_zz_old_split; /* (C+1, L) */
  double *scalars_init, *scalars_a, *scalars_b;                     /* (C+1, L, S) */
  /* moist coefficients */
  double *qtot, *cqu_e;        /* qtot (C+1, L); cqu (E+1, L) */
  double *cqw;                 /* (C+1, L+1) */
  /* vertical implicit coefficients (active rows) */
  double *cofrz;               /* (L) */
  double *cofwr, *cofwz, *cofwt, *a_tri, *alpha_tri, *gamma_tri;  /* (C, L) */
  double *coftz;               /* (C, L+1) */
  /* tendencies */
  double *tend_u, *tend_u_euler, *delsq_u;                          /* (E+1, L) */
  double *tend_w, *tend_w_euler, *tend_rw, *delsq_w;                /* (C+1, L+1) */
  double *tend_theta, *tend_theta_euler, *tend_rho, *h_divergence,
         *kdiff, *dpdz, *rthdynten, *delsq_theta, *delsq_div;       /* (C+1, L) */
  double *delsq_vort;                                               /* (V+1, L) */
  /* acoustic perturbations */
  double *ru_p;                                                     /* (E+1, L) */
  double *rw_p;                                                     /* (C+1, L+1) */
  double *rho_pp, *rtheta_pp, *rtheta_pp_old;                       /* (C+1, L) */
  /* diagnostics scratch */
  double *ke_edge;                                                  /* (E+1, L) */
  double *ke_vertex, *pv_vertex;                                    /* (V+1, L) */
  double *pv_cell;                                                  /* (C+1, L) */
  /* transport scratch */
  double *hflux;        /* (E+1, L, S)  edge high-order values / limited fluxes */
  double *flux_up, *flux_tmp;   /* (E+1, L, S) */
  double *s_max, *s_min, *scale_in, *scale_out, *rows;  /* (C+1, L, S) */
  double *wflux;        /* (C+1, L+1, S)  limiter vertical fluxes */
  double *rho_int;      /* (C+1, L) */
  /* edge-side horizontal advective fluxes of w and theta_m (one value per edge) */
  double *flux_w_e, *flux_th_e;                                     /* (E+1, L) */
  /* acoustic-step column scratch: rs / ts right-hand sides, tridiagonal rhs -> solution,
   * and the b / c diagonals of the implicit system */
  double *ac_rs, *ac_ts;                                            /* (C+1, L) */
  double *ac_x;                                                     /* (C+1, L+1) */
  double *b_tri, *c_tri;                                            /* (C+1, L) */
  double *tri_m;        /* (C+1, L) mixed form: -alpha_tri * a_tri, the forward-sweep factor */
  double *theta_edge_save;  /* (E+1, L) edge mean of theta_m_save (acoustic right-hand side) */
  double *theta_edge_rsum;  /* (E+1, L) 1 / (theta_m_save_1 + theta_m_save_2) (divergence damping) */
  /* mixed form (float32): copies of u, pv_edge, w, rw kept current by the step, the
   * deviations theta_m - ref_theta and theta_m_save - ref_theta, and the stencils'
   * intermediate edge fluxes, edge / vertex kinetic energy and vertex PV */
  float *u_f32, *pv_edge_f32, *flux_w_e_f32, *flux_th_e_f32, *ke_edge_f32;  /* (E+1, L) */
  float *w_f32, *rw_f32;                                                     /* (C+1, L+1) */
  float *theta_dev, *theta_save_dev;                                         /* (C+1, L) */
  float *pv_vertex_f32;                                                      /* (V+1, L) */
  /* status flag word (device int32[4]) for the finite check */
  int32_t *status;
} mpasg_fields;

/* ---- library info ------------------------------------------------------------- */
int mpasg_abi_version(void);
const char *mpasg_build_info(void);
/* Kernels launched by this library so far (launch accounting; graph replays excluded). */
long long mpasg_launch_count(void);

/* Stage kinds reported by mpasg_step_timed (one per recorded boundary). */
enum {
  MPASG_STAGE_BEGIN = 0, MPASG_STAGE_SETUP = 1, MPASG_STAGE_MOIST = 2, MPASG_STAGE_VIMP = 3,
  MPASG_STAGE_DYN_TEND_RK1 = 4, MPASG_STAGE_DYN_TEND = 5, MPASG_STAGE_SMLSTEP = 6,
  MPASG_STAGE_ACOUSTIC = 7, MPASG_STAGE_DIVDAMP = 8, MPASG_STAGE_RECOVER = 9,
  MPASG_STAGE_DIAG = 10, MPASG_STAGE_SPLIT = 11, MPASG_STAGE_SCALARS = 12,
  MPASG_STAGE_SCALARS_MONO = 13, MPASG_STAGE_RECONSTRUCT = 14, MPASG_STAGE_COUNT = 15
};

/* ---- whole step ----------------------------------------------------------------- */
/* Cold-start preparation: theta_m, rho_zz, ru, rw, rho_p, rtheta_*, exner*, pressure_*
 * from the loaded primitives theta (in theta_m), rho (in rho_zz) and qv (in qtot, or
 * null for dry), then diagnostics and cell-wind reconstruction. */
int mpasg_prepare(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f,
                  const double *theta, const double *rho, const double *qv, void *stream);
/* The same preparation from theta_m and rho_zz themselves (init_coupled_diagnostics.py:259:
 * the rederivation of a step boundary whose prognostics were edited); the inputs may be
 * f->theta_m and f->rho_zz. */
int mpasg_prepare_derived(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f,
                          const double *theta_m, const double *rho_zz, void *stream);
/* One large step (atm_srk3), in place on f. */
int mpasg_step(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f, void *stream);
/* The same step, recording events[i] (cudaEvent_t, timing enabled) at every stage
 * boundary and stage_kinds[i] = the MPASG_STAGE_* that ended there (i < n_events).
 * Works under stream capture (records external event nodes). Returns the number of
 * boundaries (>= 0) or a negative status. */
int mpasg_step_timed(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f,
                     void *const *events, int32_t *stage_kinds, int n_events, void *stream);
/* Autotuner: times the tile shapes of the tuned kernels on the current state (the u
 * tendency with 1, 2 and 4 levels per thread) and stores the fastest in c (tile_tend_u);
 * times_ms (optional, 3 floats) receives the measured times.  Synchronises the stream;
 * call it outside stream capture, after the state is loaded.  Leaves the state unchanged. */
int mpasg_autotune(const mpasg_mesh *m, mpasg_config *c, mpasg_fields *f, float *times_ms,
                   void *stream);
/* Applies a helper of the mixed form to n device float64 values (in -> out), for testing
 * the helpers against CUDA's own conversions and division: which = 0 float64 -> float32 ->
 * float64 through the integer repacking; which = 1 the Newton-Raphson reciprocal. */
int mpasg_numerics_check(int which, const double *in, double *out, long long n, void *stream);
/* Vector-Jacobian product of one large step's split scalar transport with explicit
 * stages (config_monotonic off, dynamics_split_steps >= 2, scalar advection on;
 * mpas_pytorch/dynamics/advance_scalars.py:1272 composed as time_integration.py:3954-4700):
 * the step's end scalars are linear in its start scalars given the step's averaged mass
 * fluxes ruavg (E+1, L) and wwavg (C+1, L+1) and the densities rho_old (at the step's
 * start) and rho_new (at its end), (C+1, L).  g_out (C+1, L, S) -> g_in (C+1, L, S).
 * adj_ptr (C+1) / adj_es: the advection stencils transposed -- for cell c, entries
 * adj_ptr[c] .. adj_ptr[c+1]-1 hold e * nAdvMax + slot of every stencil slot reading c;
 * edge_cell_w (E, 2): -edgesOnCell_sign * invAreaCell of each edge's two cells (0 for
 * the padding cell).  work: 3 (C+1) L S + (E+1) L S doubles.  The padding row of g_out passes
 * through to g_in (the step copies it unchanged).  Deterministic (gathers). */
int mpasg_transport_vjp(const mpasg_mesh *m, const mpasg_config *c, const double *ruavg,
                        const double *wwavg, const double *rho_old, const double *rho_new,
                        const int32_t *adj_ptr, const int32_t *adj_es, const double *edge_cell_w,
                        const double *g_out, double *g_in, double *work, void *stream);
/* One explicit transport stage's vector-Jacobian product (the stage of
 * mpas_pytorch/dynamics/advance_scalars.py:1272: s_out = (s_old rho_old + dt_stage (H(s_in)
 * - V(s_in))) / (w_old rho_old + w_new rho_new), fluxes ruavg / wwavg fixed): from the
 * cotangent g_out (C+1, L, S) of the stage output, writes the cotangent of s_in into the
 * active rows of g_sin and adds the cotangent of s_old into g_sold.  work_edges:
 * (E+1) L S doubles.  Used for the coupled transport mode, where every RK stage has its
 * own fluxes and density (w_old = 0, w_new = 1); adjacency arrays as for
 * mpasg_transport_vjp. */
int mpasg_transport_vjp_stage(const mpasg_mesh *m, const mpasg_config *c, double dt_stage, double w_old,
                              double w_new, const double *ruavg, const double *wwavg, const double *rho_old,
                              const double *rho_new, const int32_t *adj_ptr, const int32_t *adj_es,
                              const double *edge_cell_w, const double *g_out, double *g_sin, double *g_sold,
                              double *work_edges, void *stream);
/* One large step in two parts: part 0 runs everything but the split scalar transport
 * (the reconstruction, which reads u only, included), after which every field of the
 * step boundary but the scalars is final; part 1 runs the split transport and writes the
 * final scalars, nothing else of the boundary.  Part 0 then part 1 equals mpasg_step bit
 * for bit; the split lets a caller copy the final fields out while part 1 runs. */
int mpasg_step_part(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f, int part, void *stream);
/* One large step in the coupled transport mode (dynamics_split_steps == 1) that also
 * writes every RK stage's transport inputs into tape: for stage rk (1..3), at offset
 * (rk-1) ((E+1) L + (C+1)(L+1) + (C+1) L), ruAvg (E+1, L), wwAvg (C+1, L+1) and rho_zz
 * (C+1, L) after the stage's recovery (time_integration.py:7890-8200). */
int mpasg_step_taped(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f, double *tape, void *stream);
/* Float64 arithmetic peak of this GPU, measured: `blocks` x 256 threads each run `iters`
 * rounds of 8 independent fused multiply-adds on values read from buf (blocks * 256
 * doubles, written back so nothing is optimised away); *flops_per_s receives
 * 2 * 8 * iters * threads / time of the second of two launches.  Synchronises the stream. */
int mpasg_fp64_peak(double *buf, int blocks, int iters, double *flops_per_s, void *stream);
/* Count non-finite values of the prognostic fields into f->status[0] (async). */
int mpasg_check_finite(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f, void *stream);

/* ---- per-stage entry points (parity taps; operate on the named fields of f) ---- */
int mpasg_moist_coefficients(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f,
                             void *stream);
int mpasg_vert_imp_coefs(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f,
                         double dts, void *stream);
int mpasg_dyn_tend(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f, int rk_step,
                   void *stream);
int mpasg_smlstep_pert(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f,
                       void *stream);
int mpasg_acoustic_step(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f,
                        int small_step, double dts, void *stream);
int mpasg_divergence_damping(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f,
                             double dts, void *stream);
int mpasg_recover_large_step(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f,
                             int rk_step, int ns, double rk_dt, void *stream);
int mpasg_solve_diagnostics(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f,
                            int rk_step, void *stream);
/* Explicit RK-stage transport: scalar_old -> reads f->scalars_init, iterate f->scalars_a,
 * writes f->scalars_b; rho_zz_old = f->rho_zz_old_split, rho_zz_new = f->rho_zz,
 * fluxes f->ruAvg / f->wwAvg. */
int mpasg_advance_scalars(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f,
                          int rk_step, double dt_stage, void *stream);
int mpasg_advance_scalars_mono(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f,
                               double dt_stage, void *stream);
int mpasg_reconstruct_2d(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f,
                         void *stream);

/* ---- diagnostics outside the step ------------------------------------------------ */
/* Hydrostatic surface pressure (replaces mpas_pytorch/diagnostics.py:10
 * physics_interface_surface_pressure): rows = nCells or nCells + 1 (padding row -> 0);
 * rho_zz, zz, qv, pressure_p, pressure_base are (rows, L) row-major, zgrid (rows, L+1);
 * qv may be null (dry).  Bit-exact with the reference's float64 arithmetic. */
int mpasg_surface_pressure(int nCells, int rows, int nVertLevels, const double *rho_zz,
                           const double *zz, const double *qv, const double *pressure_p,
                           const double *pressure_base, const double *zgrid, double gravity,
                           double *out, void *stream);
/* out[0] = sum_i weight_i (x_i - ref_i)^2 over n values in a fixed summation order
 * (deterministic); ref and weight may be null (0 and 1).  The area-weighted squared
 * surface-pressure anomaly functional of the differentiation tests. */
int mpasg_weighted_sq_sum(long long n, const double *x, const double *ref, const double *weight,
                          double *out, void *stream);

/* Derivatives of mpasg_surface_pressure (the derivatives torch's autograd takes of
 * mpas_pytorch/diagnostics.py:77-82 when the reference's physics_interface_surface_pressure
 * is called on tensors that require grad), bit-identical to torch's reverse and forward
 * modes on that expression.  Shapes as mpasg_surface_pressure; qv may be null (dry).
 *   vjp: g_sp (rows) -> g_rho_zz, g_qv, g_pressure_p, g_pressure_base, each (rows, L) and
 *        fully written (levels 0 and 1 of active cells carry the derivative; other entries
 *        and the padding row are 0); any output may be null (not computed);
 *   jvp: tangents (rows, L) of the same four inputs (null = zero) -> t_sp (rows, padding
 *        row 0). */
int mpasg_surface_pressure_vjp(int nCells, int rows, int nVertLevels, const double *rho_zz,
                               const double *zz, const double *qv, const double *zgrid,
                               double gravity, const double *g_sp, double *g_rho_zz, double *g_qv,
                               double *g_pressure_p, double *g_pressure_base, void *stream);
int mpasg_surface_pressure_jvp(int nCells, int rows, int nVertLevels, const double *rho_zz,
                               const double *zz, const double *qv, const double *zgrid,
                               double gravity, const double *t_rho_zz, const double *t_qv,
                               const double *t_pressure_p, const double *t_pressure_base,
                               double *t_sp, void *stream);
/* Gradient of mpasg_weighted_sq_sum scaled by the device scalar *g_out (no host sync):
 * g_x_i = 2 ((g_out weight_i)(x_i - ref_i)), g_ref = -g_x; g_x / g_ref may be null.
 * Replaces torch's autograd through the reference-style objective
 * sum(area * (sp - sp_ref)^2) of the differentiation checks. */
int mpasg_weighted_sq_sum_vjp(long long n, const double *x, const double *ref, const double *weight,
                              const double *g_out, double *g_x, double *g_ref, void *stream);

/* ---- column tridiagonal operators and their derivatives --------------------------- */
/* One column per row: a / b / c / alpha / gamma are (n, L), rhs / out (n, L+1), float64.
 *   factor: alpha_k = 1/(b_k - a_k gamma_(k-1)), gamma_k = c_k alpha_k (k >= 1; row 0 zero)
 *   solve:  u_k = (rhs_k - a_k u_(k-1)) alpha_k (1 <= k < L); out_k = u_k - gamma_k out_(k+1)
 * *_vjp: reverse mode (gradients of every input from the output cotangents);
 * *_jvp: forward mode (output tangent from input tangents; a null tangent is zero).
 * Replace TridiagonalSolve (autodiff/tridiagonal_solve.py:177, VJP :232-291, JVP :294-352)
 * and TridiagonalFactorize (autodiff/tridiagonal_factor.py:145). */
int mpasg_tridiag_solve(long long n, int L, const double *a, const double *alpha,
                        const double *gamma, const double *rhs, double *out, void *stream);
int mpasg_tridiag_solve_vjp(long long n, int L, const double *a, const double *alpha,
                            const double *gamma, const double *rhs, const double *out,
                            const double *grad_out, double *grad_a, double *grad_alpha,
                            double *grad_gamma, double *grad_rhs, void *stream);
int mpasg_tridiag_solve_jvp(long long n, int L, const double *a, const double *alpha,
                            const double *gamma, const double *rhs, const double *out,
                            const double *da, const double *dalpha, const double *dgamma,
                            const double *drhs, double *dout, void *stream);
int mpasg_tridiag_factor(long long n, int L, const double *a, const double *b, const double *c,
                         double *alpha, double *gamma, void *stream);
int mpasg_tridiag_factor_vjp(long long n, int L, const double *a, const double *c,
                             const double *alpha, const double *gamma, const double *grad_alpha,
                             const double *grad_gamma, double *grad_a, double *grad_b,
                             double *grad_c, void *stream);
int mpasg_tridiag_factor_jvp(long long n, int L, const double *a, const double *c,
                             const double *alpha, const double *gamma, const double *da,
                             const double *db, const double *dc, double *dalpha, double *dgamma,
                             void *stream);

/* ---- dynamics derivatives (reverse mode) ------------------------------------------- */
/*
 * Hand-written vector-Jacobian products of the dry dynamics: the reverse mode the
 * reference obtains from torch autograd through atm_srk3(differentiable=True)
 * (dynamics/time_integration.py:4897-4948) and its custom Functions (dynamics/dyn_tend.py:
 * 1194,1413,1568,3860; autodiff/tridiagonal_solve.py:232-291; autodiff/tridiagonal_factor.py:
 * 183-231), with hard branches (third-order sign selectors, abs, min) frozen as taken, as in
 * autodiff/soft_limiter.py:1-10.  Cotangents live in a second mpasg_fields `g` with the same
 * layout as the forward fields: g->u is the cotangent of u, and so on.  Every transposed
 * stencil is a deterministic gather (no atomics).  Scope: float64 arithmetic, dry columns
 * (moist_end < moist_start), flat or terrain-following levels (the slope terms' upwind
 * selections sgn(flux) frozen as taken); every mixing and damping option of the
 * tendencies (2d_smagorinsky / 2d_fixed del2 and del4, vertical mixing of u, w and theta of
 * the full state or of the perturbation from the initial profiles, CAM-style top-level
 * damping, Rayleigh damping of u), the max of the CAM floor frozen as taken (a tie split
 * evenly); anything else returns MPASG_E_ARG.  The step entries (mpasg_step_tape / _vjp_taped /
 * _vjp) also take the mixed form: the tape then holds the mixed form's trajectory (its own
 * stage calls) and the reverse pass linearises it in float64.  The mass-flux averages ruAvg / wwAvg carry no
 * cotangent: they feed only the scalar transport, whose dependence on the dynamics is not
 * differentiated here.
 */
/* Transposed connectivity of one mesh (0-based; -1 where a slot has no counterpart). */
typedef struct mpasg_transpose {
  const int32_t *edgeCellSlot;   /* (E, 2) slot of the edge in edgesOnCell of cellsOnEdge[e][s] */
  const int32_t *edgeVertexSlot; /* (E, 2) slot of the edge in edgesOnVertex of verticesOnEdge[e][s] */
  const int32_t *eoeTransSlot;   /* (E, maxEdges2) slot of e in edgesOnEdge of its j-th TRiSK neighbour */
  const int32_t *cellsOnVertex;  /* (V, vertexDegree) missing -> nCells */
  const int32_t *vertexKite;     /* (V, vertexDegree) kite index (into kiteAreasOnVertex[v]) that the cell
                                    cellsOnVertex[v][s] weights this vertex with, -1 if none */
  const int32_t *advPtr;         /* (C+1) CSR: the advection-stencil slots reading each cell */
  const int32_t *advIdx;         /* e * nAdvMax + slot, in edge order */
} mpasg_transpose;

/* Doubles of the work buffer the dynamics derivatives use (any entry point below). */
long long mpasg_dyn_vjp_work_doubles(const mpasg_mesh *m);
/* Doubles of the per-step tape of mpasg_step_vjp (every RK stage's start state, the
 * dynamics-substep saves, tendencies, implicit coefficients and acoustic-substep inputs). */
long long mpasg_step_vjp_tape_doubles(const mpasg_mesh *m, const mpasg_config *c);

/* Stage VJPs.  f holds the stage's forward inputs under the names the forward entry point
 * reads; g holds the cotangents of the stage's outputs on entry and, on return, those of
 * its inputs (outputs that overwrite an input field are consumed, inputs accumulate).
 * Stages that need their forward outputs run the forward stage first, so f ends as the
 * forward stage entry point leaves it. */
/* vert_imp_coefs (vert_imp_coefs.py:188): cofwz, coftz, cofwt, a_tri, alpha_tri, gamma_tri
 * -> exner, theta_m, rtheta_p (f holds the stage's coefficients, c_tri included). */
int mpasg_vimp_vjp(const mpasg_mesh *m, const mpasg_config *c, const mpasg_fields *f, mpasg_fields *g,
                   double dts, double *work, void *stream);
/* atm_compute_dyn_tend_work (dyn_tend.py:10836): tend_u, tend_w, tend_theta, tend_rho and the
 * Euler tendencies -> u, v, w, ru, rw, ru_save, rw_save, theta_m, theta_m_save, rho_zz,
 * h_edge, divergence, vorticity, ke, pv_edge, pressure_p, rr_save (rk 1) or the rk-1
 * tendencies passed through (rk 2, 3). */
int mpasg_dyn_tend_vjp(const mpasg_mesh *m, const mpasg_config *c, const mpasg_fields *f, mpasg_fields *g,
                       const mpasg_transpose *t, int rk_step, double *work, void *stream);
/* atm_set_smlstep_pert_variables_work (smlstep_pert.py:373): tend_rw -> tend_w, tend_u. */
int mpasg_smlstep_vjp(const mpasg_mesh *m, const mpasg_config *c, const mpasg_fields *f, mpasg_fields *g,
                      void *stream);
/* atm_advance_acoustic_step_work (acoustic_step.py:1297): ru_p, rho_pp, rtheta_pp, rw_p,
 * rtheta_pp_old -> ru_p, rho_pp, rtheta_pp, rw_p (inputs), tend_u, tend_rho, tend_theta,
 * tend_rw, exner, rho_zz, w, rw, rw_save, the implicit coefficients and theta_edge_save
 * (the cotangent of the edge SUM theta_m_save_1 + theta_m_save_2).  Runs the forward
 * substep first (f's acoustic fields end as mpasg_acoustic_step leaves them). */
int mpasg_acoustic_vjp(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f, mpasg_fields *g,
                       const mpasg_transpose *t, int small_step, double dts, double *work, void *stream);
/* atm_divergence_damping_3d (divergence_damping.py:299), ru_p -> rtheta_pp, rtheta_pp_old,
 * theta_edge_save (edge-sum cotangent); f holds the stage's inputs. */
int mpasg_divdamp_vjp(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f, mpasg_fields *g,
                      double dts, double *work, void *stream);
/* atm_recover_large_step_variables_work (recover_large_step.py:1090): rho_p, rho_zz,
 * rtheta_p, theta_m, u, ru, w, rw (+ exner, pressure_p at rk 3) -> the saves and the
 * acoustic perturbations.  Runs the forward stage first. */
int mpasg_recover_vjp(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f, mpasg_fields *g,
                      int rk_step, int ns, double rk_dt, double *work, void *stream);
/* atm_compute_solve_diagnostics_work (solve_diagnostics.py:1052): h_edge, v, divergence,
 * vorticity, ke, pv_edge -> u, rho_zz, v (rk < 3).  Runs the forward stage first. */
int mpasg_diag_vjp(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f, mpasg_fields *g,
                   const mpasg_transpose *t, int rk_step, double *work, void *stream);

/* One large step's reverse sweep (the reference's per-step checkpoint with recomputation,
 * autodiff/checkpoint.py:106-254): f holds the step's start state (its 16 carried fields,
 * as mpasg_step reads them) and is advanced by one step while every RK stage's inputs are
 * written to `tape`; then the stages run backwards.  g holds the cotangents of the step's
 * end state on entry and those of its start state on return (the carried fields u, v, w,
 * ru, rw, theta_m, rho_zz, rho_p, rtheta_p, exner, pressure_p, h_edge, divergence,
 * vorticity, ke, pv_edge); g's other fields are work.  No transport, no reconstruction:
 * they do not feed the dynamics. */
int mpasg_step_vjp(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f, mpasg_fields *g,
                   const mpasg_transpose *t, double *tape, double *work, void *stream);
/* The two halves of mpasg_step_vjp, for callers that keep the tapes of several steps (no
 * recomputation, the reference's checkpoint_timesteps=False): mpasg_step_tape advances f by
 * one step writing the tape; mpasg_step_vjp_taped runs the reverse pass from a tape (f
 * supplies only the base state, moist coefficients and diabatic forcing).  g as for
 * mpasg_step_vjp. */
int mpasg_step_tape(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f, double *tape, void *stream);
/* The reverse pass of the dynamics substeps sub_lo..sub_hi (1-based) of one step, for meshes
 * whose whole-step tape does not fit: f holds the step's start state; the step is recomputed
 * up to the end of substep sub_hi with only the window taped (tape: at least
 * mpasg_step_vjp_window_tape_doubles(m, c, sub_hi - sub_lo + 1) doubles), then the window
 * runs backwards.  g holds the cotangents of the state after substep sub_hi on entry (the
 * window that ends the step: after the step) and those of the state before substep sub_lo
 * on return; calling the windows sub_hi = split .. 1 in turn, each from the restored start
 * state, gives mpasg_step_vjp's result with one substep's tape at a time.  f ends at the
 * end of substep sub_hi. */
long long mpasg_step_vjp_window_tape_doubles(const mpasg_mesh *m, const mpasg_config *c, int nsub);
int mpasg_step_vjp_window(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f, mpasg_fields *g,
                          const mpasg_transpose *t, double *tape, double *work, int sub_lo, int sub_hi,
                          void *stream);
int mpasg_step_vjp_taped(const mpasg_mesh *m, const mpasg_config *c, const mpasg_fields *f, mpasg_fields *g,
                         const mpasg_transpose *t, const double *tape, double *work, void *stream);
/* Reverse mode of the cold-start preparation (mpasg_prepare; init_coupled_diagnostics.py:147
 * and the first diagnostics): f holds the prepared state, u and w the loaded wind (edges) and
 * vertical wind (cells, L+1 levels); g the cotangents of the prepared state (consumed).
 * Writes the cotangents of the loaded u, w, theta and rho (each fully written, padding rows
 * zero). */
int mpasg_prepare_vjp(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f, mpasg_fields *g,
                      const mpasg_transpose *t, const double *w_in, double *g_u, double *g_w,
                      double *g_theta, double *g_rho, double *work, void *stream);

/* ---- dynamics derivatives (forward mode) --------------------------------------------
 * Tangents along the dynamics (the reference's run_simulation.jvp, atmosphere_model.py:2041,
 * through atm_srk3 under torch forward-mode AD), in the scope of the reverse mode above
 * (float64, dry, flat or terrain-following levels, every mixing and damping option).  d is a
 * second mpasg_fields of the same layout holding the tangents under the forward field
 * names; its padding rows hold zeros.  Every entry advances the values f through the stage
 * (as the forward entry point does) and the tangents d alongside; the branches the forward
 * takes (upwind sides, kdiff's cap, the damping layer) are frozen at the values, min ties
 * split evenly as in the reverse mode.  work: at least (nCells + 1) * (nVertLevels + 1)
 * doubles of device memory. */
/* One large step of the dynamics (no transport, no reconstruction): f and d advance. */
int mpasg_step_jvp(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f, mpasg_fields *d,
                   double *work, void *stream);
/* Tangents of the cold-start preparation (after mpasg_prepare on f): d->u and d->w hold the
 * tangents of the loaded u and w, d_theta / d_rho ((nCells+1) x L, or null for zero) those
 * of the loaded theta and rho; fills d's carried fields and diagnostics. */
int mpasg_prepare_jvp(const mpasg_mesh *m, const mpasg_config *c, const mpasg_fields *f, mpasg_fields *d,
                      const double *d_theta, const double *d_rho, void *stream);
/* Stage tangents (each stage's forward on f, tangents on d). */
int mpasg_vimp_jvp(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f, mpasg_fields *d, double dts,
                   void *stream);
int mpasg_dyn_tend_jvp(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f, mpasg_fields *d,
                       int rk_step, void *stream);
/* atm_set_smlstep_pert_variables_work (smlstep_pert.py:373) on the tangents: d's tend_w,
 * tend_u -> tend_rw; f holds the stage's inputs (its tend_u selects the terrain slope
 * coefficients; f is not written). */
int mpasg_smlstep_jvp(const mpasg_mesh *m, const mpasg_config *c, const mpasg_fields *f, mpasg_fields *d,
                      void *stream);
int mpasg_acoustic_jvp(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f, mpasg_fields *d,
                       int small_step, double dts, double *work, void *stream);
int mpasg_divdamp_jvp(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f, mpasg_fields *d, double dts,
                      void *stream);
int mpasg_recover_jvp(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f, mpasg_fields *d,
                      int rk_step, int ns, double rk_dt, void *stream);
int mpasg_diag_jvp(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f, mpasg_fields *d, int rk_step,
                   void *stream);

/* ---- boundary binding ----------------------------------------------------------- */
/* 128-bit value digest of nbytes bytes at p (device memory, 8-byte aligned) into out[0..1]
 * (device memory): the lanes A = sum h_i and B = sum mix(h_i ^ 0x5851f42d4c957f2d) modulo
 * 2^64 over the little-endian 8-byte words w_i (last word zero-padded), h_i = mix(w_i ^
 * mix(i + 0x9e3779b97f4a7c15)), mix = the SplitMix64 output function.  Independent of the
 * summation order.  Binds a returned step boundary to its values (the reference keeps the
 * bytes themselves, state.py:72-141 mark_complete_step_boundary). */
int mpasg_digest(const void *p, long long nbytes, unsigned long long *out, void *stream);

/* ---- mesh reordering (host functions; no GPU needed) -------------------------------- */
/* new_to_old[i] = the old index of the i-th point along the 3-D Hilbert curve through
 * the points (x, y, z) (cell or vertex centres).  Replaces the reference's RCM orders
 * (mpas_pytorch/mesh_reordering.py:44-79) with a space-filling-curve order. */
int mpasg_sfc_order(long long n, const double *x, const double *y, const double *z,
                    long long *new_to_old);
/* Edge order of the reference's rule (mesh_reordering.py:82-103): sort by (min, max) of
 * the edge's new 1-based cell ids (missing cells -> n_cells + 1), then old index.
 * cells_on_edge is (n_edges, 2) 1-based; cell_old_to_new 0-based. */
int mpasg_edge_order(long long n_edges, long long n_cells, const long long *cells_on_edge,
                     const long long *cell_old_to_new, long long *new_to_old);

/* Device row gather for reordered meshes: dst[i, :] = src[rows[i], :] for i < n, rows of
 * row_len float64 values (rows: device int64).  src and dst must not overlap. */
int mpasg_permute_rows(const double *src, double *dst, const long long *rows, long long n,
                       long long row_len, void *stream);

/* ---- transport without caller scratch -------------------------------------------- */
/* Capacity (float64 values) of the library-owned edge scratch: nEdges * L * S must not
 * exceed it (32 MiB; e.g. 30720 edges x 41 levels x 3 scalars fits). */
#define MPASG_STATIC_SCRATCH_DOUBLES (1 << 22)
/*
 * mpasg_advance_scalars_static: the same explicit RK-stage transport as
 * mpasg_advance_scalars (same fields read and written, same results bit for bit), but
 * its per-edge scratch (f->hflux in the other entry point) is a fixed array inside the
 * library, so f->hflux may be null and the call allocates and borrows nothing.
 * No counterpart in the reference: its atm_advance_scalars_work
 * (dynamics/advance_scalars.py:1272) allocates its work tensors on every call.
 *
 * For callers that can hand over only the stage's own arrays (scalar_old/new, rho_zz
 * old/new, uhAvg, wwAvg) and may not allocate device memory themselves: e.g. a host
 * model whose device memory is owned by its own pool, or one that may not call an
 * allocator inside its time loop.
 *
 *  - The first call on each device looks up the scratch address (and may load the
 *    module); make that first call, with that device current, before any stream capture.
 *    The address is cached for the life of the device's primary context: after a
 *    cudaDeviceReset the cached address is stale, so do not call this entry point on that
 *    device again in the same process.
 *  - Returns MPASG_E_SCRATCH, launching nothing, when nEdges * L * S exceeds
 *    MPASG_STATIC_SCRATCH_DOUBLES.
 *  - No scratch value needs to start at zero: each call writes every entry it reads.
 *  - There is one scratch per device: calls that overlap on one device (other streams,
 *    other threads) race on it. Order them (one stream, or events between streams).
 */
int mpasg_advance_scalars_static(const mpasg_mesh *m, const mpasg_config *c, mpasg_fields *f,
                                 int rk_step, double dt_stage, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* MPASG_H */
