/*
 * gckpp_gb300.h -- C ABI of the GB300 KPP fullchem chemistry solve.
 *
 * A drop-in for the per-cell chemistry loop of GEOS-Chem's Do_FullChem
 * (GeosCore/fullchem_mod.F90:528-1551).  Where the reference calls, once per
 * grid cell and OpenMP thread,
 *
 *     CALL Update_RCONST()                                  ! fullchem_mod.F90:953
 *     CALL Integrate( 0.0_dp, DT, ICNTRL, RCNTRL,
 *                     ISTATUS, RSTATE, IERR )               ! fullchem_mod.F90:1033
 *
 * on thread-private module globals (C, RCONST, ATOL/RTOL: KPP/fullchem/
 * gckpp_Global.F90:47-128), a caller of this library hands over a batch of
 * cells at once.  Every per-cell array is cell-interleaved ("structure of
 * arrays"): element k of cell i is at X[k*ld + i] with ld >= ncell, which is
 * what a Fortran caller gets from an array declared X(ld, K) and indexed
 * X(cell, k).  Species, reaction and ISTATUS/RSTATUS indices are 0-based
 * here; index k here is index k+1 in the reference's Fortran.
 *
 * All entry points are plain C, take plain pointers and sizes, never abort
 * and never print.  They return 0 on success or a negative GC_KPP_E* code;
 * gc_kpp_last_error() describes the last failure of the calling thread.
 * Per-cell integrator errors are not call failures: they are reported in
 * ierr[] with the reference's IERR codes (1 = success, -1 ... -8 as in
 * ros_ErrorMsg, KPP/fullchem/gckpp_Integrator.F90:538-575).
 */
#ifndef GCKPP_GB300_H
#define GCKPP_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* call status codes */
#define GC_KPP_OK 0
#define GC_KPP_EINVAL (-101)      /* bad argument */
#define GC_KPP_ECUDA (-102)       /* CUDA runtime error */
#define GC_KPP_ENOMEM (-103)      /* device allocation failed */
#define GC_KPP_EUNSUPPORTED (-104) /* option outside the implemented path */

/* where the caller's arrays live */
#define GC_KPP_MEM_HOST 0
#define GC_KPP_MEM_DEVICE 1

/* gc_kpp_ctx_set_option keys */
#define GC_KPP_OPT_ARITH 1        /* 0 = fast (FMA, reciprocal pivots), 1 = strict (reference order, no FMA),
                                     2 = fast with 2 cells per thread, 3 = fast with 4 cells per thread
                                     (0 and 1 integrate 1 cell per thread) */
#define GC_KPP_OPT_SCHEDULE 2     /* 0 = plain (thread per cell), 1 = persistent work queue */
#define GC_KPP_OPT_BLOCK 3        /* threads per block (multiple of 32, <= 1024), 0 = default 128 */
#define GC_KPP_OPT_BLOCKS_PER_SM 4 /* queue schedule: resident blocks per SM, 0 = default */
#define GC_KPP_OPT_MAX_SLOTS 5    /* cap on workspace slots (cells in flight), 0 = no cap */
#define GC_KPP_OPT_TIMING 6       /* 1 = time the Rosenbrock launches with CUDA events */
#define GC_KPP_OPT_LU 7           /* 0 = row-wise LU (default), 1 = KppDecomp right-looking order */
#define GC_KPP_OPT_CELL_BLOCK 8   /* threads of the block-per-cell kernel (multiple of 32, <= 1024),
                                     0 = default 256; 32 is one warp per cell */
#define GC_KPP_OPT_EVICT_AFTER 10 /* > 0: a cell of the thread-per-cell queue that still runs after
                                     this many steps is handed over, at a step boundary, to the
                                     block-per-cell kernel, which finishes it with the same
                                     arithmetic (same results with GC_KPP_OPT_BLOCK_SPLIT 0);
                                     0 = off (default).  Needs the queue
                                     schedule, ARITH 0 or 1, the row-wise LU and ISTATUS/RSTATUS
                                     arrays (the fullchem step always has them). */
#define GC_KPP_OPT_EVICT_DRAINED 11 /* 1 = hand a cell over only once the work queue has no
                                       unclaimed cell left (the tail of the launch); 0 = as soon
                                       as it has taken GC_KPP_OPT_EVICT_AFTER steps (default) */
#define GC_KPP_OPT_BLOCK_SPLIT 12 /* fast arithmetic (ARITH 0, 2, 3): 1 = the block-per-cell kernel
                                     runs the split form (default): 256 threads, every sum of the
                                     LU, the substitutions, Fun_SPLIT and Jac_SP cut into chunks
                                     that the lanes of a warp segment add in a shuffle tree, which
                                     shortens the serial chains of a stiff cell's step; results
                                     agree with the thread-per-cell form to rounding.  0 = the
                                     level form (GC_KPP_OPT_CELL_BLOCK threads, each sum in one
                                     thread, results identical to the thread-per-cell form). */
#define GC_KPP_OPT_RATES_DIRECT 13 /* 1 = Update_RCONST runs as straight-line code generated
                                      from the mechanism's rate program (default); 0 = the
                                      rate-program interpreter.  The same operations in the
                                      same order; results agree to rounding (within 1e-13
                                      relative: compile-time constants let the compiler
                                      specialise a few libm calls). */
#define GC_KPP_OPT_QUEUE_CHUNK 14 /* queue schedule: queue positions a lane of the thread-per-cell
                                      kernel takes per claim, in [1, 64]; 0 = default 1.  A lane
                                      integrates its positions one after the other and claims
                                      again when they are used up (the chunk of an OpenMP
                                      SCHEDULE(DYNAMIC, chunk) cell loop).  Results do not
                                      depend on it. */
#define GC_KPP_OPT_ASYNC 9        /* 1 = chemistry steps never synchronise the host, so that a
                                     caller can capture them in a CUDA graph: the retry list and
                                     the block-per-cell count stay on the device, *nretry (and
                                     *nblock of the learned step) are set to -1.  Needs device
                                     memory, the queue schedule, and tolerance arrays that a
                                     synchronous step on this context has checked; make one
                                     synchronous call of the largest batch before capturing
                                     (buffers are sized then, never inside a capture). */

/* Per-cell meteorology/state fields of gc_kpp_update_rconst_batch (rows of
 * `met`), the thread-private globals that Set_Kpp_GridBox_Values and the
 * sulfur/cloud routines fill before Update_RCONST
 * (GeosCore/fullchem_mod.F90:2089-2167, KPP/fullchem/commonIncludeVars.H). */
#define GC_KPP_MET_TEMP 0      /* TEMP [K] */
#define GC_KPP_MET_NUMDEN 1    /* NUMDEN, air number density [molec/cm3] */
#define GC_KPP_MET_H2O 2       /* H2O [molec/cm3] */
#define GC_KPP_MET_PRESS 3     /* PRESS [hPa] */
#define GC_KPP_MET_SRHOCL 4    /* SRHOCl [cm3/molec/s] */
#define GC_KPP_MET_SRHOBR 5    /* SRHOBr [cm3/molec/s] */
#define GC_KPP_MET_K_MT 6      /* K_MT(1:6), rows 6..11 */
#define GC_KPP_MET_K_CLD 12    /* K_CLD(1:6), rows 12..17 */
#define GC_KPP_NMET 18
#define GC_KPP_NPHOTOL 200     /* PHOTOL(1:200) rows */

typedef struct gc_kpp_ctx gc_kpp_ctx;

/* Mechanism dimensions (NSPEC, NVAR, NFIX, NREACT, LU_NONZERO of
 * KPP/fullchem/gckpp_Parameters.F90:34-54).  Any pointer may be NULL. */
int gc_kpp_mechanism_dims(int* nspec, int* nvar, int* nfix, int* nreact, int* lu_nonzero);

/* Create a solver context on CUDA device `device`: uploads the mechanism
 * tables.  Workspace is allocated on first use and grown as needed.
 * Replaces nothing in the reference (its state is module globals). */
int gc_kpp_ctx_create(gc_kpp_ctx** ctx, int device);
int gc_kpp_ctx_destroy(gc_kpp_ctx* ctx);
int gc_kpp_ctx_set_option(gc_kpp_ctx* ctx, int key, long long value);

/* Message for the last failed call on this thread ("" if none). */
const char* gc_kpp_last_error(void);

/* Batched INTEGRATE (KPP/fullchem/gckpp_Integrator.F90:80-162) over ncell
 * independent cells, from TIN to TOUT.
 *
 *   c        [NSPEC][ldc]  in/out  concentrations (molec/cm3); variable
 *                                  species are integrated, fixed ones read
 *   rconst   [NREACT][ldr] in      rate constants from Update_RCONST
 *   atol,rtol [NVAR]       in      tolerances (ICNTRL(2)=0) or [1] (scalar)
 *   icntrl   [20], rcntrl [20]     as ICNTRL_U/RCNTRL_U of INTEGRATE; zero
 *                                  ICNTRL entries and non-positive RCNTRL
 *                                  entries keep the defaults (:112-117)
 *   hstart   [ncell] or NULL       per-cell RCNTRL(3) (the KPPHvalue chain,
 *                                  fullchem_AutoReduceFuncs.F90:287)
 *   istatus  [20][ldo] out or NULL ISTATUS(1:8) counters, rest zero
 *   rstatus  [20][ldo] out or NULL RSTATUS(1:3) = Texit, Hexit, Hnew;
 *                                  RSTATUS(4) = auto-reduce threshold
 *                                  with a target species, rest zero
 *   ierr     [ncell]   out         IERR per cell
 *   mem      GC_KPP_MEM_HOST or GC_KPP_MEM_DEVICE for all arrays above
 *   stream   cudaStream_t (NULL = default stream); with device memory the
 *            call is asynchronous on that stream, with host memory it
 *            returns after the results are copied back.
 *
 * Supported: Rosenbrock methods ICNTRL(3) = 0..6, autonomous or not,
 * vector or scalar tolerances, ICNTRL(4) step cap, ICNTRL(16) clamping,
 * RCNTRL(1:7), and auto-reduction (ICNTRL(12) = 1: ros_yIntegrator,
 * :789-1237; with ICNTRL(13) = 1 the append form ros_yIntegratorA,
 * :1242-1700) with threshold RCNTRL(12) (default 100 molec/cm3/s) or a
 * target species ICNTRL(14) in 1..NVAR with ratio RCNTRL(14), the
 * threshold then reported in RSTATUS(4).  Auto-reduction runs on the
 * thread-per-cell kernel with GC_KPP_OPT_ARITH 0 or 1 and the row-wise LU.
 * GC_KPP_EUNSUPPORTED for: in-integrator rate updates (ICNTRL(15) must be
 * -1, 0 after merging, or 2), a target species outside VAR, and
 * auto-reduction with more cells per thread or the KppDecomp-order LU. */
int gc_kpp_integrate_batch(gc_kpp_ctx* ctx, int ncell, double tin, double tout,
                           double* c, long long ldc,
                           const double* rconst, long long ldr,
                           const double* atol, const double* rtol,
                           const int* icntrl, const double* rcntrl,
                           const double* hstart,
                           int* istatus, double* rstatus, long long ldo,
                           int* ierr, int mem, void* stream);

/* Batched Update_RCONST (KPP/fullchem/gckpp_Rates.F90:408-1503): the 1058
 * rate constants of each cell from its met state.
 *
 *   met     [GC_KPP_NMET][ldm]    in   fields GC_KPP_MET_*
 *   photol  [GC_KPP_NPHOTOL][ldp] in   J-values PHOTOL(1:200) [1/s]
 *   c       [NSPEC][ldc]          in   concentrations (read by uptake rates)
 *   rconst  [NREACT][ldr]         out  RCONST
 *
 * Gas-phase, photolysis, K_MT/K_CLD and constant rates are evaluated as the
 * reference does.  Heterogeneous rates are 0 (no aerosol surface, no cloud);
 * gc_kpp_update_rconst_het_batch evaluates them from a HetState. */
int gc_kpp_update_rconst_batch(gc_kpp_ctx* ctx, int ncell, const double* met, long long ldm,
                               const double* photol, long long ldp, const double* c, long long ldc,
                               double* rconst, long long ldr, int mem, void* stream);

/* Rows of the HetState array of gc_kpp_update_rconst_het_batch: the fields
 * of the reference's HetState type (KPP/fullchem/commonIncludeVars.H:111-201)
 * in declaration order, one row per scalar and one per array element
 * (aWater 2, KHETI_SLA 11, pHSSA 2, wetArea/xArea/xH2O/xRadi/xVol 14 each,
 * logicals as 0.0/1.0), then SUNCOS; 168 rows.  Row offsets: the HET_*
 * macros of geos-chem_gb300/csrc/het_layout.h. */
#define GC_KPP_NHET 168

/* gc_kpp_update_rconst_batch with the cells' HetState (replaces the
 * State_Het that fullchem_SetStateHet fills before Update_RCONST,
 * GeosCore/fullchem_mod.F90:861-936):
 *
 *   het     [GC_KPP_NHET][ldh]    in   HetState rows (NULL: heterogeneous rates 0)
 *
 * The heterogeneous rates are the fullchem rate laws of
 * KPP/fullchem/fullchem_RateLawFuncs.F90:795-3460 (uptake on aerosol types,
 * cloud droplets and ice, with kIIR1Ltd's limiting-reactant form and
 * CloudHet's entrainment limit), reading C, MW/SR_MW/HENRY_K0/HENRY_CR of the
 * species database and RELHUM from TEMP and H2O as Set_Kpp_GridBox_Values
 * computes it.  Mechanisms other than fullchem keep their heterogeneous
 * rates at 0. */
/* Rows of the grid-box input array of gc_kpp_set_state_het_batch,
 * gc_kpp_sulfur_aq_rates_batch, gc_kpp_sulfur_cld_rates_batch and
 * gc_kpp_het_drop_chem_batch: the
 * State_Met and State_Chm fields of the grid box that fullchem_SetStateHet,
 * fullchem_SulfurAqChem and SET_SO2 read, in their units (T, CLDF, QI, QL,
 * AIRVOL, AIRDEN, AD, FRLAND, FROCEAN, InStratosphere, aClArea, aClRadi,
 * IsorropAeroH2O(2), AeroArea(14), AeroRadi(14), WetAeroArea(14),
 * AeroH2O(14), OMOC_POA, OMOC_OPOA, HSO3_aq, SO3_aq, IsorropBisulfate,
 * IsorropNitrate, IsorropSulfate, IsorropHplus, pHCloud, IsorropAeropH(2),
 * the sea-salt species SALA, SALAAL, SALC, SALCAL [molec/cm3],
 * fupdateHOBr, fupdateHOCl, KHETI_SLA(11), STATE_PSC), then SUNCOS, then
 * SET_SO2's PMID_DRY [hPa] and the non-KPP species NH4, NH3, DSTbin1..7,
 * pFe [molec/cm3], then HetDropChem's OMEGA [Pa/s], U, V [m/s] and IsWater
 * (0/1); 115 rows.  Row offsets: the HETIN_* macros of
 * geos-chem_gb300/csrc/het_layout.h. */
#define GC_KPP_NHETIN 115

/* Batched fullChem_SetStateHet (KPP/fullchem/fullchem_HetStateFuncs.F90:
 * 48-244, with Cld_Params, Get_Theta_Ice and Halide_Conc; called at
 * GeosCore/fullchem_mod.F90:885): the HetState rows of each cell.
 *
 *   hetin  [GC_KPP_NHETIN][ldi]  in   grid-box fields (rows above)
 *   c      [NSPEC][ldc]          in   KPP concentrations (SO2, HNO3, HCl, HBr,
 *                                     BrSALA, BrSALC, SALACL, SALCCL, NIT,
 *                                     NITs, SO4 are read)
 *   gamma_ho2, lpscchem, turn_off_het_rates
 *                                     Input_Opt%gamma_HO2, %LPSCCHEM (0/1),
 *                                     %TurnOffHetRates (0/1)
 *   het    [GC_KPP_NHET][ldh]    out  HetState rows, SUNCOS copied from hetin
 *
 * Fields the reference routine does not set (H2O, and the Hg-only cloudBox,
 * fracOrgAer, fracInorgAer) are written as 0. */
int gc_kpp_set_state_het_batch(gc_kpp_ctx* ctx, int ncell, const double* hetin, long long ldi,
                               const double* c, long long ldc, double gamma_ho2, int lpscchem,
                               int turn_off_het_rates, double* het, long long ldh, int mem, void* stream);

/* Batched fullchem_SulfurAqChem (KPP/fullchem/fullchem_SulfurChemFuncs.F90:
 * 120-305, called from Set_Sulfur_Chem_Rates at GeosCore/fullchem_mod.F90:
 * 861): K_MT(1:6), the uptake of SO2 (by O3), HCl and HNO3 on alkaline fine
 * and coarse sea salt, from the wet area and radius of aerosol types 11 and
 * 12 (AeroArea/WetAeroArea/AeroRadi rows of hetin) and C(SALAAL), C(SALCAL),
 * C(O3), C(SO2), C(HCl), C(HNO3) -- C as fullchem_ConvertAlkToEquiv leaves
 * it before the call (SALAAL and SALCAL times MW * 7e-5, fullchem_mod.F90's
 * Set_Sulfur_Chem_Rates; the caller converts them, and back after the solve).
 *
 *   met  [GC_KPP_NMET][ldm]  in/out  TEMP and NUMDEN read; the six K_MT rows
 *                                     (GC_KPP_MET_K_MT..+5) written, the
 *                                     other rows untouched */
int gc_kpp_sulfur_aq_rates_batch(gc_kpp_ctx* ctx, int ncell, const double* hetin, long long ldi,
                                 const double* c, long long ldc, double* met, long long ldm, int mem,
                                 void* stream);

/* Batched fullchem_SulfurCldChem, i.e. SET_SO2
 * (KPP/fullchem/fullchem_SulfurChemFuncs.F90:320-398 and 865-1620, with
 * GET_HPLUS :1635-1853, its equilibrium functions :1867-3156 and AQCHEM_SO2
 * :3171-3549; called from Set_Sulfur_Chem_Rates at GeosCore/fullchem_mod.F90:
 * 861 after fullchem_SulfurAqChem): for cloudy cells (CLDF > 1e-4,
 * T > 258 K, in-cloud liquid water > 1e-20, SO2 present) the cloud water's
 * pH by Newton's method on its electroneutrality, then K_CLD(1:6), the
 * aqueous oxidation of S(IV) by H2O2, O3, O2 (metal catalysed, when
 * lmetalcatso2 = Input_Opt%LMETALCATSO2 = 1) and HCHO and the HMS rates.
 *
 *   hetin [GC_KPP_NHETIN][ldi] in/out  grid-box fields (rows above); the
 *                                      HSO3_aq, SO3_aq and pHCloud rows are
 *                                      overwritten (1e-32, 1e-32, 0 outside
 *                                      cloud) and fupdateHOBr/HOCl set to 1,
 *                                      as Set_Sulfur_Chem_Rates leaves them
 *                                      for fullchem_SetStateHet
 *   c     [NSPEC][ldc]  in            KPP concentrations (SO2, H2O2, O3,
 *                                      CH2O, SO4, SO4s, HMS, SALACL, SALCCL,
 *                                      HCl, HCOOH, ACTA, HNO3, NIT, NITs read)
 *   met   [GC_KPP_NMET][ldm] in/out   the six K_CLD rows (GC_KPP_MET_K_CLD..
 *                                      +5) written, the other rows untouched
 *   size_res [ncell] out or NULL       1 where the reference would call
 *                                      fullchem_HetDropChem (not built here)
 *
 * Where the reference stops the model (a NaN pH), the cell's pHCloud and
 * K_CLD come out NaN. */
int gc_kpp_sulfur_cld_rates_batch(gc_kpp_ctx* ctx, int ncell, double* hetin, long long ldi, const double* c,
                                  long long ldc, double* met, long long ldm, int lmetalcatso2, int* size_res,
                                  int mem, void* stream);

/* Batched fullchem_HetDropChem (KPP/fullchem/fullchem_SulfurChemFuncs.F90:
 * 414-790) with Do_FullChem's call conditions (GeosCore/fullchem_mod.F90:
 * 913-934: CLDF > 1e-4, size_res from gc_kpp_sulfur_cld_rates_batch, the
 * IsWater row set, TEMP > 268.15 K, in-cloud liquid water > 1e-20): the
 * size-resolved cloud-droplet oxidation of S(IV) by HOCl and HOBr (Yuen et
 * al. 1996) as the rate coefficients SRHOCl and SRHOBr, which the step's
 * HOCl + SO2 and HOBr + SO2 rates add (0 where the conditions fail, as
 * fullchem_mod.F90:575-577 resets them).  Call after
 * gc_kpp_set_state_het_batch: the sulfite uptake laws read its HetState.
 *
 *   dt       chemistry time step [s]
 *   hetin    [GC_KPP_NHETIN][ldi] in  grid-box rows after SET_SO2 (HSO3_aq,
 *                                     SO3_aq, CLDF, QL, AIRDEN, AD, AIRVOL,
 *                                     NH3, SALC, OMEGA, U, V, IsWater read)
 *   c        [NSPEC][ldc] in          SO2, H2O2, O3, HOCl, HOBr, HNO3, SO4
 *   het      [GC_KPP_NHET][ldh] in    HetState rows
 *   size_res [ncell] in
 *   met      [GC_KPP_NMET][ldm] in/out TEMP, NUMDEN, H2O, PRESS, K_CLD(1:3)
 *                                     read; the SRHOCL and SRHOBR rows written */
int gc_kpp_het_drop_chem_batch(gc_kpp_ctx* ctx, int ncell, double dt, const double* hetin, long long ldi,
                               const double* c, long long ldc, const double* het, long long ldh, const int* size_res,
                               double* met, long long ldm, int mem, void* stream);

/* HetState of the cells of the following chemistry steps on this context
 * (gc_kpp_fullchem_step and its ordered/binned/learned forms evaluate the
 * heterogeneous rates from it): het [GC_KPP_NHET][ldh] for `ncell` cells, in
 * device memory (kept by pointer: the caller keeps it alive and up to date)
 * or host memory (copied now).  het = NULL clears it (heterogeneous rates 0).
 * A step over a different number of cells fails with GC_KPP_EINVAL. */
int gc_kpp_ctx_set_hetstate(gc_kpp_ctx* ctx, int ncell, const double* het, long long ldh, int mem);

/* Auto-reduction controls of the following integrations with ICNTRL(12) = 1
 * on this context, as Do_FullChem sets them per grid box
 * (KPP/fullchem/fullchem_AutoReduceFuncs.F90:274-343, GeosCore/
 * fullchem_mod.F90:510-515 and :585-587):
 *
 *   thr    [ncell] or NULL  RCNTRL(12) of each cell (<= 0: the default 100)
 *   target [ncell] or NULL  ICNTRL(14) of each cell, 0..NVAR (1-based
 *                           species; 0 = threshold mode)
 *   ratio  [ncell] or NULL  RCNTRL(14) of each cell (<= 0: 0)
 *   keep   [NVAR]  or NULL  keepSpcActive in HOST memory: nonzero species
 *                           are never frozen (keepActive on); NULL = off
 *   mem    GC_KPP_MEM_HOST or GC_KPP_MEM_DEVICE for thr/target/ratio
 *
 * The arrays are copied.  A NULL per-cell array leaves that control to the
 * call's ICNTRL/RCNTRL.  Each call replaces every earlier setting; all NULL
 * clears them.  An integration over a different number of cells (the cell
 * count, or cell_limit of the ordered forms) fails with GC_KPP_EINVAL; a
 * target outside 0..NVAR fails here with GC_KPP_EUNSUPPORTED.  Integrations
 * without ICNTRL(12) = 1 ignore these controls. */
int gc_kpp_ctx_set_autoreduce(gc_kpp_ctx* ctx, int ncell, const double* thr, const int* target,
                              const double* ratio, const unsigned char* keep, int mem);

int gc_kpp_update_rconst_het_batch(gc_kpp_ctx* ctx, int ncell, const double* met, long long ldm,
                                   const double* photol, long long ldp, const double* c, long long ldc,
                                   const double* het, long long ldh, double* rconst, long long ldr, int mem,
                                   void* stream);

/* One chemistry step of Do_FullChem's cell loop for a batch of cells
 * (GeosCore/fullchem_mod.F90:528-1551, the loop body from :817 to :1350):
 *   zero the prod/loss family dummies (:943-946), Update_RCONST (:953),
 *   save C (:1023), Integrate(0, DT) with RCNTRL(3) = hstart[cell] (:1033),
 *   for cells with IERR < 0 integrate once more from the saved C with
 *   Hstart = 0 (:1138-1162), hstart[cell] = RSTATE(Nhnew) (:1294), and
 *   C = MAX(C, 0) (:1329-1350).
 *
 *   met/photol   as gc_kpp_update_rconst_batch
 *   c            [NSPEC][ldc] in/out
 *   hstart       [ncell] in/out or NULL: the KPPHvalue chain
 *   istatus/rstatus/ierr as gc_kpp_integrate_batch (the final attempt)
 *   nretry       out or NULL: number of cells integrated a second time
 * A cell that fails twice keeps IERR < 0; like the reference with KppStop
 * off, its concentrations are those of the failed attempt, clamped. */
int gc_kpp_fullchem_step(gc_kpp_ctx* ctx, int ncell, double dt, const double* met, long long ldm,
                         const double* photol, long long ldp, double* c, long long ldc,
                         const double* atol, const double* rtol, const int* icntrl, const double* rcntrl,
                         double* hstart, int* istatus, double* rstatus, long long ldo, int* ierr,
                         int* nretry, int mem, void* stream);

/* gc_kpp_fullchem_step with a queue order: order[0..ncell-1] is a
 * permutation of the cells, the order in which the persistent work-queue
 * schedule starts them (GC_KPP_OPT_SCHEDULE = 1; the plain schedule assigns
 * order[i] to thread slot i).  Each cell's integration is independent of
 * the others, so the results are those of gc_kpp_fullchem_step for any
 * order; the order changes only how the work packs onto the GPU.  Starting
 * the cells that need the most steps first keeps a few stiff cells from
 * running alone at the end of the launch.  No counterpart in the reference
 * (its OpenMP loop hands out chunks of 24 cells in grid order,
 * SCHEDULE(DYNAMIC, 24), fullchem_mod.F90:528-545).  With host memory the
 * order is checked to be a permutation (GC_KPP_EINVAL otherwise); with
 * device memory, entries outside [0, ncell) are skipped and their cells
 * left untouched. */
int gc_kpp_fullchem_step_ordered(gc_kpp_ctx* ctx, int ncell, double dt, const double* met, long long ldm,
                                 const double* photol, long long ldp, double* c, long long ldc,
                                 const double* atol, const double* rtol, const int* icntrl, const double* rcntrl,
                                 double* hstart, int* istatus, double* rstatus, long long ldo, int* ierr,
                                 int* nretry, const int* order, int mem, void* stream);

/* gc_kpp_fullchem_step_ordered in which the first nblock cells of `order`
 * are integrated block-per-cell: all threads of a block (GC_KPP_OPT_CELL_BLOCK)
 * work on one cell whose Jacobian, LU factors and stage vectors are held in
 * shared memory, on a second stream beside the thread-per-cell queue that
 * takes the other cells.  Meant for the few stiff cells that need tens of
 * steps while most need one or two; each cell gets the same arithmetic in
 * either form (to rounding in the split form, GC_KPP_OPT_BLOCK_SPLIT).
 * Needs GC_KPP_OPT_ARITH 0 or 1 and the row-wise LU
 * (GC_KPP_EUNSUPPORTED otherwise).  No counterpart in the reference. */
int gc_kpp_fullchem_step_binned(gc_kpp_ctx* ctx, int ncell, double dt, const double* met, long long ldm,
                                const double* photol, long long ldp, double* c, long long ldc,
                                const double* atol, const double* rtol, const int* icntrl, const double* rcntrl,
                                double* hstart, int* istatus, double* rstatus, long long ldo, int* ierr,
                                int* nretry, const int* order, int nblock, int mem, void* stream);

/* The learned proposer on the device: the MLP of the learned step-size /
 * stiffness proposer (56 -> 128 -> 128 -> 5, GELU; include/gckpp_gb300_mlp.h
 * has its kernels), created from host arrays: w1 [128][56], w2 [128][128],
 * w3 [5][128] (rounded to BF16 on upload), biases b1 [128], b2 [128], b3 [5],
 * the feature normalisation mean/inv_std [56], the PHOTOL rows jrows [20] and
 * species rows srows [32] of the features, and scale: H0 = scale *
 * exp(out[0]).  No counterpart in the reference. */
typedef struct gc_kpp_proposer gc_kpp_proposer;
int gc_kpp_proposer_create(int device, const float* w1, const float* b1, const float* w2, const float* b2,
                           const float* w3, const float* b3, const double* mean, const double* inv_std,
                           const int* jrows, const int* srows, double scale, gc_kpp_proposer** proposer);
int gc_kpp_proposer_destroy(gc_kpp_proposer* proposer);
/* Largest H0 the proposer proposes [s] (cap > 0; 0 restores the default, the
 * chemistry step's length).  A cap keeps the first step of a cold-started
 * cell near the sizes the plain integration reaches on its own, which holds
 * the learned step's error to the plain step's.  No counterpart in the
 * reference. */
int gc_kpp_proposer_set_h0_cap(gc_kpp_proposer* proposer, double cap);

/* gc_kpp_fullchem_step with the learned plan in front: features of every
 * cell, the MLP, H0 proposals written into hstart where it is not positive
 * (cells without a KPPHvalue; clamped to [1e-5, min(dt, H0 cap)]), stiffness bins, the
 * stable heaviest-bin-first queue order, and gc_kpp_fullchem_step_binned
 * with the top bin block-per-cell (*nblock receives its size).  Same
 * arguments and results as gc_kpp_fullchem_step; with device memory, hstart
 * is required (zeros for a cold start).  The error-controlled integration
 * decides every step: the proposals change the work, not the tolerance. */
int gc_kpp_fullchem_step_learned(gc_kpp_ctx* ctx, gc_kpp_proposer* proposer, int ncell, double dt,
                                 const double* met, long long ldm, const double* photol, long long ldp, double* c,
                                 long long ldc, const double* atol, const double* rtol, const int* icntrl,
                                 const double* rcntrl, double* hstart, int* istatus, double* rstatus,
                                 long long ldo, int* ierr, int* nretry, int* nblock, int mem, void* stream);

/* Batched INTEGRATE that allocates nothing, for callers that cannot call
 * cudaMalloc: an embedding framework or host model that owns all device
 * memory through its own pool, or a process whose allocator must not be
 * touched in the middle of a time step.  No counterpart in the reference
 * (whose state is module globals); arguments and results are those of
 * gc_kpp_integrate_batch, with every array in device memory and the fast
 * arithmetic with one thread per cell.  Auto-reduction (ICNTRL(12) = 1) is
 * refused with GC_KPP_EUNSUPPORTED.  The call reads ATOL/RTOL back to the
 * host for the tolerance check and waits for that copy on the stream.
 *
 * It needs no context: its workspace for at most GC_KPP_NOALLOC_MAX_CELLS
 * cells (about 157 MB) and its copy of the mechanism tables are file-scope
 * device arrays of the library, held by every GPU that loads it until the
 * process exits.  Larger batches are rejected with GC_KPP_EINVAL: split them.
 * The first call on a device sets it up (copies the tables in and looks up
 * the device addresses, with that device current), so make that first call
 * before any stream capture.  All calls on a device share its one workspace:
 * calls that overlap on the GPU (issued on different streams or from
 * different host threads) race and must be serialised by the caller.  The
 * workspace keeps the last call's contents; nothing in it needs to start at
 * zero, since every entry a call reads it has written first. */
#define GC_KPP_NOALLOC_MAX_CELLS 1024
int gc_kpp_integrate_batch_noalloc(int ncell, double tin, double tout, double* c, long long ldc,
                                   const double* rconst, long long ldr, const double* atol,
                                   const double* rtol, const int* icntrl, const double* rcntrl,
                                   const double* hstart, int* istatus, double* rstatus, long long ldo,
                                   int* ierr, void* stream);

/* Number of kernels the last gc_kpp_fullchem_step call on ctx launched. */
int gc_kpp_last_launch_count(gc_kpp_ctx* ctx);

/* With GC_KPP_OPT_TIMING set: device time [ms] of the Rosenbrock kernel
 * launches of the last integrate/step call (waits for them to finish). */
int gc_kpp_last_kernel_ms(gc_kpp_ctx* ctx, double* ms, int* nlaunch);

/* Stream-ordered copy of `rows` rows of `width` bytes from src (row pitch
 * spitch bytes) to dst (row pitch dpitch), each side in host or device
 * memory of the current device.  Page-locked host memory (cudaHostAlloc,
 * cudaHostRegister) is read and written by the GPU's SMs through its device
 * alias; pageable host memory goes through cudaMemcpy2DAsync.  The
 * library's own host-memory calls stage their arrays this way: on GB300,
 * after a chemistry step a copy engine needs ~60-90 ms for the first 1 GB of
 * a page-locked buffer and the SMs ~5-10 ms.  No counterpart in the
 * reference (its arrays never leave the host). */
int gc_kpp_copy_rows(void* dst, long long dpitch, const void* src, long long spitch, long long width, long long rows,
                     void* stream);

/* mask[r] = 1 for the GC_KPP_NPHOTOL rows r of PHOTOL that the mechanism's
 * Update_RCONST reads (168 of 200 for fullchem), 0 for the others, which a
 * caller need not send; host-memory steps copy only these rows.  No
 * counterpart in the reference. */
int gc_kpp_photol_rows(unsigned char* mask);

#ifdef __cplusplus
}
#endif

#endif /* GCKPP_GB300_H */
