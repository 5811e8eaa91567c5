/*
 * swm_oracle.h -- CPU restatement of the SWM time-stepping hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the
 * GB300 kernels: only tests/, __graft_entry__.smoke() and the cpu_baseline
 * leg of bench.py may load it.  The product path never links it.
 *
 * Every routine restates one Fortran routine of martinclaus/swm (file:line
 * cited at the definition in swm_oracle.c), in FP64, with the reference's
 * evaluation order kept so that results agree to the last bit where the
 * reference's own arithmetic is deterministic.
 *
 * Layout: every 2-D field is Fortran column-major (Nx, Ny), i.e. C row-major
 * [Ny][Nx] with i fastest; indices are 0-based here.
 */
#ifndef SWM_ORACLE_H
#define SWM_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  ORC_MODE_NONE = 0,       /* no linearisation define (selfcheck test1 layout)   */
  ORC_MODE_NONLINEAR = 1,  /* FULLY_NONLINEAR                                    */
  ORC_MODE_LIN_REST = 2,   /* LINEARISED_STATE_OF_REST                           */
  ORC_MODE_LIN_MEAN = 3    /* LINEARISED_MEAN_STATE                              */
};

enum { ORC_MIX_LAPLACE = 0, ORC_MIX_BIHARMONIC = 1 };

typedef struct orc_config {
  int32_t nx, ny;
  int32_t mode;
  int32_t lateral_mixing;      /* LATERAL_MIXING                       */
  int32_t quadratic_friction;  /* QUADRATIC_BOTTOM_FRICTION            */
  int32_t barotropic;          /* BAROTROPIC                           */
  int32_t mixing_kind;         /* ORC_MIX_*; biharmonic is a project extension */
  int32_t coriolis_approx;     /* 0 none, 1 f-plane, 2 beta-plane, 3 sphere */
  int32_t tracer_nan_guard;    /* extension: 0/0 tracer coefficients -> 0 */
  int32_t damping_additive;    /* fixture compat: damping entries add up (see orc_damping_add) */
  int32_t mask_psi_bs;         /* fixture compat: basic-state psi zeroed on land H points */
  int32_t tracer_flux;         /* 0 reference centred flux; 1 third-order upwind-biased (extension) */
  int32_t frozen_flow;         /* extension: SWM state held fixed, only tracers step */
  double dt, G, Ah, A, OMEGA, RHO0, lbc, theta0;
  double lon_s, lon_e, lat_s, lat_e;
  double H_overwrite;          /* 0 = not set (H_OVERWRITE_DEF)        */
  double ab_chi, minD;
  double tau_scale;            /* 1.0 when TAU_SCALE is undefined      */
  double bih;                  /* biharmonic coefficient (extension)   */
} orc_config;

typedef struct orc_model orc_model;

/* field ids for orc_field() */
enum {
  ORC_U0, ORC_U1, ORC_V0, ORC_V1, ORC_ETA0, ORC_ETA1,
  ORC_GU1, ORC_GU2, ORC_GU3, ORC_GV1, ORC_GV2, ORC_GV3, ORC_GETA1, ORC_GETA2, ORC_GETA3,
  ORC_D, ORC_DH, ORC_DU, ORC_DV, ORC_EDENS, ORC_POT, ORC_ZETA, ORC_MU, ORC_MV,
  ORC_H, ORC_HU, ORC_HV, ORC_HETA,
  ORC_IMPL_U, ORC_IMPL_V, ORC_IMPL_ETA, ORC_GSQ_U, ORC_GSQ_V,
  ORC_GLIN_U, ORC_GLIN_V, ORC_GLIN_ETA,
  ORC_FX, ORC_FY, ORC_FETA, ORC_FX_CONST, ORC_FY_CONST, ORC_FETA_CONST,
  ORC_U_BS, ORC_V_BS, ORC_ZETA_BS, ORC_PSI_BS,
  ORC_LATMIX_U, ORC_LATMIX_V, ORC_PLL, ORC_PLT,
  ORC_TOT_U, ORC_TOT_V, ORC_TOT_ETA,
  ORC_BC_H, ORC_BC_U, ORC_BC_V, ORC_BC_ETA,
  ORC_NFIELDS
};
/* 1-D (Ny) metric ids for orc_lat() */
enum {
  ORC_LAT_H, ORC_LAT_U, ORC_LAT_V, ORC_LAT_ETA,
  ORC_COS_H, ORC_COS_U, ORC_COS_V, ORC_COS_ETA,
  ORC_TAN_H, ORC_TAN_U, ORC_TAN_V, ORC_TAN_ETA,
  ORC_F_H, ORC_F_U, ORC_F_V, ORC_F_ETA,
  ORC_NLAT
};
enum { ORC_OCEAN_H, ORC_OCEAN_U, ORC_OCEAN_V, ORC_OCEAN_ETA };

/* damping namelist entry kinds (swm_damping_nl) */
enum { ORC_TERM_GLIN_U, ORC_TERM_GLIN_V, ORC_TERM_GLIN_ETA, ORC_TERM_GSQ_U, ORC_TERM_GSQ_V };
enum { ORC_DAMP_UNIFORM, ORC_DAMP_SPONGE, ORC_DAMP_FILE };
enum { ORC_SPONGE_N = 1, ORC_SPONGE_S = 2, ORC_SPONGE_W = 4, ORC_SPONGE_E = 8 };

/* forcing stream kinds (swm_forcing_nl forcingtype / component first letter) */
enum { ORC_FRC_WIND, ORC_FRC_OSC, ORC_FRC_CUSTOM, ORC_FRC_HEAT, ORC_FRC_EMF };
enum { ORC_CMP_ZONAL, ORC_CMP_MERID, ORC_CMP_CONT, ORC_CMP_U2, ORC_CMP_V2, ORC_CMP_REY };

/* ---- domain / grid (initDomain) ---- */
orc_model *orc_create(const orc_config *cfg, const double *H_in, const int8_t *H_missing);
void orc_destroy(orc_model *m);
double *orc_field(orc_model *m, int id);
double *orc_lat(orc_model *m, int id);
int8_t *orc_ocean(orc_model *m, int id);
void orc_get_scalars(const orc_model *m, double *dLambda, double *dTheta);
void orc_set_itt(orc_model *m, int64_t itt);
int64_t orc_get_itt(const orc_model *m);

/* ---- SWM init sequence (SWM_initSWM) ---- */
void orc_set_psi_bs(orc_model *m, const double *psi);
void orc_timestep_init(orc_model *m);
void orc_damping_add(orc_model *m, int term, int type, double value, double sl_length,
                     double sl_cutoff, int locflags, const double *file_data);
void orc_damping_finalize(orc_model *m);
int orc_forcing_add_stream(orc_model *m, int type, int component, double omega,
                           int is_constant, const double *d1, const double *d2);
void orc_forcing_set_data(orc_model *m, int stream, const double *d1, const double *d2);
void orc_forcing_init(orc_model *m);
void orc_forcing_update(orc_model *m);
void orc_initial_conditions(orc_model *m, const double *eta, const double *u, const double *v);

/* ---- time loop (model.f90 timestepModel) ---- */
void orc_swm_timestep(orc_model *m);   /* SWM_timestep */
void orc_swm_advance(orc_model *m);    /* SWM_advance   */
void orc_model_advance(orc_model *m);  /* model_advance (totals reset + SWM_advance + TRC_advance) */
void orc_run(orc_model *m, int64_t nsteps); /* itt+1 .. itt+nsteps with steady forcing */

/* ---- diagnostics helpers (calc_lib) ---- */
void orc_streamfunction(orc_model *m, const double *u, const double *v, double *psi);
void orc_divergence(orc_model *m, const double *u, const double *v, double *div);
void orc_nondivergent_from_chi(orc_model *m, const double *chi, const double *u, const double *v, double *u_nd,
                               double *v_nd);

/* ---- tracer (tracer_module / tracer_vars) ---- */
int orc_tracer_add(orc_model *m, double kappa_h, double cons, double gamma_c,
                   const double *C, const double *C0, const double *gamma_field,
                   const double *cons_field);
void orc_tracer_init(orc_model *m);       /* TRC_initCoeffs */
double *orc_tracer_field(orc_model *m, int tracer, int id);
enum { ORC_TRC_CH0, ORC_TRC_CH1, ORC_TRC_G1, ORC_TRC_G2, ORC_TRC_G3, ORC_TRC_C, ORC_TRC_C0,
       ORC_TRC_GAMMA, ORC_TRC_IMPL, ORC_TRC_UHC, ORC_TRC_VHC, ORC_TRC_DIFF, ORC_TRC_FORCING,
       ORC_TRC_NFIELDS };
void orc_tracer_timestep(orc_model *m);   /* TRC_timestep */
void orc_tracer_advance(orc_model *m);    /* TRC_advance  */
double *orc_tracer_coeff(orc_model *m);   /* TRC_coeff (12, Nx, Ny) */

/* ---- red-black SOR (ElSolv_SOR) ---- */
void orc_sor_init(orc_model *m);
int orc_sor_solve(orc_model *m, const double *B, double *chi, double eps, int first_guess,
                  double *anorm_out);
const double *orc_sor_coeff(orc_model *m); /* ElSolvSOR_c (Nx, Ny, 5) */

/* ---- extension: variable-coefficient Helmholtz red-black SOR (standalone) ---- */
void orc_helmholtz_coeffs(int nx, int ny, const double *hinv, double lambda, double dx, double dy, double *cx,
                          double *cy, double *cc);
int orc_helmholtz_sor(int nx, int ny, const double *cx, const double *cy, const double *cc,
                      const int8_t *mask, const double *rhs, double *psi, double omega,
                      double rtol, int max_sweeps, double *relres_out);
void orc_helmholtz_apply(int nx, int ny, const double *cx, const double *cy, const double *cc,
                         const int8_t *mask, const double *psi, double *out);

#ifdef __cplusplus
}
#endif
#endif
