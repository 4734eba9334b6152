/* CPU oracle of the KPP fullchem Rosenbrock solve -- TEST INFRASTRUCTURE.
 *
 * A plain-C restatement of the reference's per-cell integration
 * (KPP/fullchem/gckpp_Integrator.F90, gckpp_LinearAlgebra.F90) used only by
 * the tests, the smoke check and the CPU-baseline leg of the benchmark, to
 * check or time against.  It is never linked into, or called by, the product
 * library.
 */
#ifndef KPP_ORACLE_H
#define KPP_ORACLE_H
#include "kpp_dims.h" /* generated per mechanism (oracle/_gen/<mechanism>/) */

extern const int ORACLE_LU_CROW[];
extern const int ORACLE_LU_DIAG[];
extern const int ORACLE_LU_ICOL[];
extern const int ORACLE_LU_IROW[];

void oracle_fun_split(const double* V, const double* F, const double* RCT, double* Vdot);
void oracle_jac_sp(const double* V, const double* F, const double* RCT, double* JVS);
void oracle_kpp_solve(const double* JVS, double* X);
void oracle_kpp_solve_slv(const double* JVS, double* X, const unsigned char* DO_SLV);
void oracle_fun_pd(const double* V, const double* F, const double* RCT, double* P, double* D);
int oracle_kpp_decomp(double* JVS);

/* Update_RCONST for one cell.  met[18] = TEMP, NUMDEN, H2O, PRESS, SRHOCl,
 * SRHOBr, K_MT(1:6), K_CLD(1:6); PHOTOL[200]; C[NSPEC]. */
void oracle_update_rconst(const double* met, const double* PHOTOL, const double* C, double* RCONST);
void oracle_update_rconst_batch(int ncell, const double* met, long long ldm, const double* photol, long long ldp,
                                const double* c, long long ldc, double* rconst, long long ldr);
/* The same with the cells' HetState rows het[f * ldh + cell] (NULL: zeroed
 * HetState), for the heterogeneous rate laws of het_laws.h. */
void oracle_update_rconst_het(const double* met, const double* PHOTOL, const double* C, const double* het,
                              long long ldh, double* RCONST);
void oracle_update_rconst_het_batch(int ncell, const double* met, long long ldm, const double* photol,
                                    long long ldp, const double* c, long long ldc, const double* het, long long ldh,
                                    double* rconst, long long ldr);

/* One cell: INTEGRATE(TIN, TOUT, ICNTRL_U, RCNTRL_U, ISTATUS, RSTATUS, IERR)
 * on C[NSPEC] (in/out) with RCONST[NREACT]. */
void oracle_integrate(double* C, const double* RCONST, const double* atol, const double* rtol,
                      double tin, double tout, const int* icntrl_u, const double* rcntrl_u,
                      int* istatus, double* rstatus, int* ierr);

/* Batch over cells in the cell-interleaved layout X[k*ld + cell], OpenMP
 * SCHEDULE(DYNAMIC,24) like the reference loop (fullchem_mod.F90:528-543).
 * hstart (optional) is the per-cell RCNTRL(3). */
void oracle_integrate_batch(int ncell, double tin, double tout, double* c, long long ldc,
                            const double* rconst, long long ldr, const double* atol, const double* rtol,
                            const int* icntrl_u, const double* rcntrl_u, const double* hstart,
                            int* istatus, double* rstatus, long long ldo, int* ierr, int nthreads);
/* The same with per-cell RCNTRL(12), ICNTRL(14), RCNTRL(14) (each optional). */
void oracle_integrate_batch_ar(int ncell, double tin, double tout, double* c, long long ldc,
                               const double* rconst, long long ldr, const double* atol, const double* rtol,
                               const int* icntrl_u, const double* rcntrl_u, const double* hstart,
                               int* istatus, double* rstatus, long long ldo, int* ierr, int nthreads,
                               const double* ar_thr, const int* ar_target, const double* ar_ratio);
/* keepSpcActive [NVAR] (nonzero = never frozen) with keepActive on; NULL
 * turns keepActive off. */
void oracle_set_keep(const unsigned char* keep);
int oracle_max_threads(void);
#endif
