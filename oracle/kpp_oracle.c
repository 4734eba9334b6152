/* CPU oracle: restatement of the KPP Rosenbrock integrator -- TEST INFRASTRUCTURE.
 *
 * Follows, routine by routine (paths relative to the GEOS-Chem source root):
 *   INTEGRATE              KPP/fullchem/gckpp_Integrator.F90:80-162
 *   Rosenbrock (setup)     KPP/fullchem/gckpp_Integrator.F90:165-532
 *   ros_Integrator         KPP/fullchem/gckpp_Integrator.F90:578-786
 *   ros_ErrorNorm          KPP/fullchem/gckpp_Integrator.F90:1715-1745
 *   ros_FunTimeDerivative  KPP/fullchem/gckpp_Integrator.F90:1748-1769
 *   ros_PrepareMatrix      KPP/fullchem/gckpp_Integrator.F90:1921-1999
 *   ros_Decomp/ros_Solve   KPP/fullchem/gckpp_Integrator.F90:2003-2057
 *   method coefficients    KPP/fullchem/gckpp_Integrator.F90:2060-2480
 *   KppDecomp              KPP/fullchem/gckpp_LinearAlgebra.F90:46-83
 *   WAXPY / WSCAL          KPP/fullchem/gckpp_LinearAlgebra.F90:3762-3858
 *   WLAMCH('E')            KPP/fullchem/gckpp_LinearAlgebra.F90:3861-3905
 *   FunTemplate/JacTemplate KPP/fullchem/gckpp_Integrator.F90:2487-2621
 *
 * Fortran MIN/MAX are restated with fmin/fmax: a NaN operand yields the other
 * operand (the reference leaves that case compiler-defined).
 * Compiled with -ffp-contract=off this performs the reference's arithmetic.
 */
#include "kpp_oracle.h"

#include <float.h>
#include <math.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NVAR ORACLE_NVAR
#define NSPEC ORACLE_NSPEC
#define NREACT ORACLE_NREACT
#define LU_NONZERO ORACLE_LU_NONZERO

/* ISTATUS / RSTATUS slots (0-based) */
enum { Nfun = 0, Njac, Nstp, Nacc, Nrej, Ndec, Nsol, Nsng };
enum { Ntexit = 0, Nhexit, Nhnew };

int oracle_kpp_decomp(double* JVS) {
  double W[NVAR];
  double a;
  int k, kk, j, jj;
  for (k = 0; k < NVAR; ++k) {
    if (fabs(JVS[ORACLE_LU_DIAG[k]]) < DBL_MIN) return k + 1;
    for (kk = ORACLE_LU_CROW[k]; kk < ORACLE_LU_CROW[k + 1]; ++kk) W[ORACLE_LU_ICOL[kk]] = JVS[kk];
    for (kk = ORACLE_LU_CROW[k]; kk < ORACLE_LU_DIAG[k]; ++kk) {
      j = ORACLE_LU_ICOL[kk];
      a = -W[j] / JVS[ORACLE_LU_DIAG[j]];
      W[j] = -a;
      for (jj = ORACLE_LU_DIAG[j] + 1; jj < ORACLE_LU_CROW[j + 1]; ++jj)
        W[ORACLE_LU_ICOL[jj]] = W[ORACLE_LU_ICOL[jj]] + a * JVS[jj];
    }
    for (kk = ORACLE_LU_CROW[k]; kk < ORACLE_LU_CROW[k + 1]; ++kk) JVS[kk] = W[ORACLE_LU_ICOL[kk]];
  }
  return 0;
}

static void waxpy(int n, double alpha, const double* x, double* y) {
  if (alpha == 0.0) return;
  for (int i = 0; i < n; ++i) y[i] = y[i] + alpha * x[i];
}

static void wscal(int n, double alpha, double* x) {
  if (alpha == 1.0) return;
  for (int i = 0; i < n; ++i) {
    if (alpha == -1.0) x[i] = -x[i];
    else if (alpha == 0.0) x[i] = 0.0;
    else x[i] = alpha * x[i];
  }
}

static double wlamch_e(void) {
  volatile double eps = pow(0.5, 16), suma;
  for (int i = 17; i <= 80; ++i) {
    eps = eps * 0.5;
    suma = 1.0 + eps;
    if (suma <= 1.0) return eps * 2.0;
  }
  return eps;
}

typedef struct {
  int S;
  double A[15], C[15], M[6], E[6], Alpha[6], Gamma[6], ELO;
  int NewF[6];
} method_t;

static int method_init(int id, method_t* r) {
  memset(r, 0, sizeof(*r));
  if (id == 1) { /* Ros2 */
    double g = 1.0 + 1.0 / sqrt(2.0);
    r->S = 2; r->A[0] = 1.0 / g; r->C[0] = -2.0 / g; r->NewF[0] = r->NewF[1] = 1;
    r->M[0] = 3.0 / (2.0 * g); r->M[1] = 1.0 / (2.0 * g);
    r->E[0] = 1.0 / (2.0 * g); r->E[1] = 1.0 / (2.0 * g);
    r->ELO = 2.0; r->Alpha[1] = 1.0; r->Gamma[0] = g; r->Gamma[1] = -g;
  } else if (id == 2) { /* Ros3 */
    r->S = 3; r->A[0] = 1.0; r->A[1] = 1.0; r->A[2] = 0.0;
    r->C[0] = -0.10156171083877702091975600115545E+01;
    r->C[1] = 0.40759956452537699824805835358067E+01;
    r->C[2] = 0.92076794298330791242156818474003E+01;
    r->NewF[0] = 1; r->NewF[1] = 1; r->NewF[2] = 0;
    r->M[0] = 0.1E+01; r->M[1] = 0.61697947043828245592553615689730E+01;
    r->M[2] = -0.42772256543218573326238373806514;
    r->E[0] = 0.5; r->E[1] = -0.29079558716805469821718236208017E+01;
    r->E[2] = 0.22354069897811569627360909276199;
    r->ELO = 3.0;
    r->Alpha[1] = r->Alpha[2] = 0.43586652150845899941601945119356;
    r->Gamma[0] = 0.43586652150845899941601945119356;
    r->Gamma[1] = 0.24291996454816804366592249683314;
    r->Gamma[2] = 0.21851380027664058511513169485832E+01;
  } else if (id == 3) { /* Ros4 */
    r->S = 4;
    r->A[0] = 0.2000000000000000E+01; r->A[1] = 0.1867943637803922E+01; r->A[2] = 0.2344449711399156;
    r->A[3] = r->A[1]; r->A[4] = r->A[2]; r->A[5] = 0.0;
    r->C[0] = -0.7137615036412310E+01; r->C[1] = 0.2580708087951457E+01; r->C[2] = 0.6515950076447975;
    r->C[3] = -0.2137148994382534E+01; r->C[4] = -0.3214669691237626; r->C[5] = -0.6949742501781779;
    r->NewF[0] = r->NewF[1] = r->NewF[2] = 1; r->NewF[3] = 0;
    r->M[0] = 0.2255570073418735E+01; r->M[1] = 0.2870493262186792; r->M[2] = 0.4353179431840180;
    r->M[3] = 0.1093502252409163E+01;
    r->E[0] = -0.2815431932141155; r->E[1] = -0.7276199124938920E-01; r->E[2] = -0.1082196201495311;
    r->E[3] = -0.1093502252409163E+01;
    r->ELO = 4.0;
    r->Alpha[1] = 0.1145640000000000E+01; r->Alpha[2] = 0.6552168638155900; r->Alpha[3] = r->Alpha[2];
    r->Gamma[0] = 0.5728200000000000; r->Gamma[1] = -0.1769193891319233E+01;
    r->Gamma[2] = 0.7592633437920482; r->Gamma[3] = -0.1049021087100450;
  } else if (id == 0 || id == 4) { /* Rodas3 */
    r->S = 4;
    r->A[1] = 2.0; r->A[3] = 2.0; r->A[5] = 1.0;
    r->C[0] = 4.0; r->C[1] = 1.0; r->C[2] = -1.0; r->C[3] = 1.0; r->C[4] = -1.0; r->C[5] = -(8.0 / 3.0);
    r->NewF[0] = 1; r->NewF[1] = 0; r->NewF[2] = 1; r->NewF[3] = 1;
    r->M[0] = 2.0; r->M[1] = 0.0; r->M[2] = 1.0; r->M[3] = 1.0;
    r->E[3] = 1.0;
    r->ELO = 3.0;
    r->Alpha[2] = 1.0; r->Alpha[3] = 1.0;
    r->Gamma[0] = 0.5; r->Gamma[1] = 1.5;
  } else if (id == 5) { /* Rodas4 */
    r->S = 6;
    r->Alpha[1] = 0.386; r->Alpha[2] = 0.210; r->Alpha[3] = 0.630; r->Alpha[4] = 1.000; r->Alpha[5] = 1.000;
    r->Gamma[0] = 0.2500000000000000; r->Gamma[1] = -0.1043000000000000; r->Gamma[2] = 0.1035000000000000;
    r->Gamma[3] = -0.3620000000000023E-01;
    r->A[0] = 0.1544000000000000E+01; r->A[1] = 0.9466785280815826; r->A[2] = 0.2557011698983284;
    r->A[3] = 0.3314825187068521E+01; r->A[4] = 0.2896124015972201E+01; r->A[5] = 0.9986419139977817;
    r->A[6] = 0.1221224509226641E+01; r->A[7] = 0.6019134481288629E+01; r->A[8] = 0.1253708332932087E+02;
    r->A[9] = -0.6878860361058950;
    r->A[10] = r->A[6]; r->A[11] = r->A[7]; r->A[12] = r->A[8]; r->A[13] = r->A[9]; r->A[14] = 1.0;
    r->C[0] = -0.5668800000000000E+01; r->C[1] = -0.2430093356833875E+01; r->C[2] = -0.2063599157091915;
    r->C[3] = -0.1073529058151375; r->C[4] = -0.9594562251023355E+01; r->C[5] = -0.2047028614809616E+02;
    r->C[6] = 0.7496443313967647E+01; r->C[7] = -0.1024680431464352E+02; r->C[8] = -0.3399990352819905E+02;
    r->C[9] = 0.1170890893206160E+02; r->C[10] = 0.8083246795921522E+01; r->C[11] = -0.7981132988064893E+01;
    r->C[12] = -0.3152159432874371E+02; r->C[13] = 0.1631930543123136E+02; r->C[14] = -0.6058818238834054E+01;
    r->M[0] = r->A[6]; r->M[1] = r->A[7]; r->M[2] = r->A[8]; r->M[3] = r->A[9]; r->M[4] = 1.0; r->M[5] = 1.0;
    r->E[5] = 1.0;
    for (int i = 0; i < 6; ++i) r->NewF[i] = 1;
    r->ELO = 4.0;
  } else if (id == 6) { /* Rang3 */
    r->S = 4;
    r->A[0] = 5.09052051067020e+00; r->A[1] = 5.09052051067020e+00; r->A[2] = 0.0;
    r->A[3] = 4.97628111010787e+00; r->A[4] = 2.77268164715849e-02; r->A[5] = 2.29428036027904e-01;
    r->C[0] = -1.16790812312283e+01; r->C[1] = -1.64057326467367e+01; r->C[2] = -2.77268164715850e-01;
    r->C[3] = -8.38103960500476e+00; r->C[4] = -8.48328409199343e-01; r->C[5] = 2.87009860433106e-01;
    r->M[0] = 5.22582761233094e+00; r->M[1] = -5.56971148154165e-01; r->M[2] = 3.57979469353645e-01;
    r->M[3] = 1.72337398521064e+00;
    r->E[0] = -5.16845212784040e+00; r->E[1] = -1.26351942603842e+00; r->E[2] = -1.11022302462516e-16;
    r->E[3] = 2.22044604925031e-16;
    r->Alpha[1] = 2.21878746765329e+00; r->Alpha[2] = 2.21878746765329e+00; r->Alpha[3] = 1.55392337535788e+00;
    r->Gamma[0] = 4.35866521508459e-01; r->Gamma[1] = -1.78292094614483e+00;
    r->Gamma[2] = -2.46541900496934e+00; r->Gamma[3] = -8.05529997906370e-01;
    for (int i = 0; i < 4; ++i) r->NewF[i] = 1;
    r->ELO = 3.0;
  } else {
    return 0;
  }
  return 1;
}

typedef struct {
  const double* fix;
  const double* rct;
  int istatus[20];
  double rstatus[20];
} cellctx_t;

static void fun_template(cellctx_t* cx, const double* y, double* ydot) {
  oracle_fun_split(y, cx->fix, cx->rct, ydot);
}
static void jac_template(cellctx_t* cx, const double* y, double* jcb) {
  oracle_jac_sp(y, cx->fix, cx->rct, jcb);
}

static double error_norm(const double* Y, const double* Ynew, const double* Yerr, const double* AbsTol,
                         const double* RelTol, int VectorTol) {
  double Err = 0.0, Scale, Ymax;
  for (int i = 0; i < NVAR; ++i) {
    Ymax = fmax(fabs(Y[i]), fabs(Ynew[i]));
    if (VectorTol) Scale = AbsTol[i] + RelTol[i] * Ymax;
    else Scale = AbsTol[0] + RelTol[0] * Ymax;
    double q = Yerr[i] / Scale;
    Err = Err + q * q;
  }
  Err = sqrt(Err / NVAR);
  return fmax(Err, 1.0e-10);
}

static void fun_time_derivative(cellctx_t* cx, double T, double Roundoff, const double* Y, const double* Fcn0,
                                double* dFdT) {
  const double DeltaMin = 1.0e-6;
  double Delta = sqrt(Roundoff) * fmax(DeltaMin, fabs(T));
  (void)T;
  fun_template(cx, Y, dFdT); /* rates frozen: FunTemplate(T+Delta) == Fun(Y) */
  cx->istatus[Nfun] += 1;
  waxpy(NVAR, -1.0, Fcn0, dFdT);
  wscal(NVAR, 1.0 / Delta, dFdT);
}

static void prepare_matrix(cellctx_t* cx, double* H, int Direction, double gam, const double* Jac0, double* Ghimj,
                           int* Singular) {
  int Nconsecutive = 0;
  *Singular = 1;
  while (*Singular) {
    for (int i = 0; i < LU_NONZERO; ++i) Ghimj[i] = -Jac0[i];
    double ghinv = 1.0 / (Direction * (*H) * gam);
    for (int i = 0; i < NVAR; ++i) Ghimj[ORACLE_LU_DIAG[i]] = Ghimj[ORACLE_LU_DIAG[i]] + ghinv;
    int ising = oracle_kpp_decomp(Ghimj);
    cx->istatus[Ndec] += 1;
    if (ising == 0) {
      *Singular = 0;
    } else {
      cx->istatus[Nsng] += 1;
      Nconsecutive += 1;
      *Singular = 1;
      if (Nconsecutive <= 5) *H = (*H) * 0.5;
      else return;
    }
  }
}

static void ros_integrator(cellctx_t* cx, const method_t* m, double* Y, double Tstart, double Tend, double* Tout,
                           const double* AbsTol, const double* RelTol, int Autonomous, int VectorTol,
                           int Max_no_steps, double Roundoff, double Hmin, double Hmax, double Hstart, double FacMin,
                           double FacMax, double FacRej, double FacSafe, int clamp, int* IERR) {
  double Ynew[NVAR], Fcn0[NVAR], Fcn[NVAR], K[6 * NVAR], dFdT[NVAR], Yerr[NVAR];
  static __thread double Jac0[LU_NONZERO], Ghimj[LU_NONZERO];
  double H, Hnew, HC, HG, Fac, Err;
  int Direction, ioffset, j, istage, RejectLastH, RejectMoreH, Singular;
  const double DeltaMin = 1.0e-5;
  double T = Tstart;
  cx->rstatus[Nhexit] = 0.0;
  H = fmin(fmax(fabs(Hmin), fabs(Hstart)), fabs(Hmax));
  if (fabs(H) <= 10.0 * Roundoff) H = DeltaMin;
  Direction = (Tend >= Tstart) ? +1 : -1;
  H = Direction * H;
  RejectLastH = 0;
  RejectMoreH = 0;
  memset(dFdT, 0, sizeof(dFdT));

  while ((Direction > 0 && ((T - Tend) + Roundoff <= 0.0)) || (Direction < 0 && ((Tend - T) + Roundoff <= 0.0))) {
    if (cx->istatus[Nstp] > Max_no_steps) { *IERR = -6; *Tout = T; return; }
    if (((T + 0.1 * H) == T) || (H <= Roundoff)) { *IERR = -7; *Tout = T; return; }
    H = fmin(H, fabs(Tend - T));
    fun_template(cx, Y, Fcn0);
    cx->istatus[Nfun] += 1;
    if (!Autonomous) fun_time_derivative(cx, T, Roundoff, Y, Fcn0, dFdT);
    jac_template(cx, Y, Jac0);
    cx->istatus[Njac] += 1;
    for (;;) { /* UntilAccepted */
      prepare_matrix(cx, &H, Direction, m->Gamma[0], Jac0, Ghimj, &Singular);
      if (Singular) { *IERR = -8; *Tout = T; return; }
      for (istage = 1; istage <= m->S; ++istage) {
        ioffset = NVAR * (istage - 1);
        if (istage == 1) {
          memcpy(Fcn, Fcn0, sizeof(Fcn));
        } else if (m->NewF[istage - 1]) {
          memcpy(Ynew, Y, sizeof(Ynew));
          for (j = 1; j <= istage - 1; ++j)
            waxpy(NVAR, m->A[(istage - 1) * (istage - 2) / 2 + j - 1], K + NVAR * (j - 1), Ynew);
          fun_template(cx, Ynew, Fcn);
          cx->istatus[Nfun] += 1;
        }
        memcpy(K + ioffset, Fcn, sizeof(Fcn));
        for (j = 1; j <= istage - 1; ++j) {
          HC = m->C[(istage - 1) * (istage - 2) / 2 + j - 1] / (Direction * H);
          waxpy(NVAR, HC, K + NVAR * (j - 1), K + ioffset);
        }
        if (!Autonomous && m->Gamma[istage - 1] != 0.0) {
          HG = Direction * H * m->Gamma[istage - 1];
          waxpy(NVAR, HG, dFdT, K + ioffset);
        }
        oracle_kpp_solve(Ghimj, K + ioffset);
        cx->istatus[Nsol] += 1;
      }
      memcpy(Ynew, Y, sizeof(Ynew));
      for (j = 1; j <= m->S; ++j) waxpy(NVAR, m->M[j - 1], K + NVAR * (j - 1), Ynew);
      memset(Yerr, 0, sizeof(Yerr));
      for (j = 1; j <= m->S; ++j) waxpy(NVAR, m->E[j - 1], K + NVAR * (j - 1), Yerr);
      Err = error_norm(Y, Ynew, Yerr, AbsTol, RelTol, VectorTol);
      Fac = fmin(FacMax, fmax(FacMin, FacSafe / pow(Err, 1.0 / m->ELO)));
      Hnew = H * Fac;
      cx->istatus[Nstp] += 1;
      if ((Err <= 1.0) || (H <= Hmin)) {
        cx->istatus[Nacc] += 1;
        if (clamp) for (int i = 0; i < NVAR; ++i) Y[i] = fmax(Ynew[i], 0.0);
        else memcpy(Y, Ynew, sizeof(Ynew));
        T = T + Direction * H;
        Hnew = fmax(Hmin, fmin(Hnew, Hmax));
        if (RejectLastH) Hnew = fmin(Hnew, H);
        cx->rstatus[Nhexit] = H;
        cx->rstatus[Nhnew] = Hnew;
        cx->rstatus[Ntexit] = T;
        RejectLastH = 0;
        RejectMoreH = 0;
        H = Hnew;
        break;
      } else {
        if (RejectMoreH) Hnew = H * FacRej;
        RejectMoreH = RejectLastH;
        RejectLastH = 1;
        H = Hnew;
        if (cx->istatus[Nacc] >= 1) cx->istatus[Nrej] += 1;
      }
    }
  }
  *Tout = T;
  *IERR = 1;
}

/* ---- auto-reduce (gckpp_Integrator.F90:789-1237, 1702-1712, 2624-2661) ----
 * ros_yIntegrator: at the first step the species whose production and loss
 * (Fun_SPLITF's P_VAR and D_VAR*y) are both below the threshold are frozen
 * (DO_SLV false); the others are integrated with the Jacobian restricted to
 * them (compressed pattern cLU_*, cKppDecomp) and KppSolve's DO_SLV-guarded
 * statements; at the end each frozen species takes the first-order
 * solution y = P/k + (y - P/k) exp(-k dt) (AutoReduce_1stOrder).
 * ros_yIntegratorA (:1242-1700) adds APPEND (:2663-2700): at every step a
 * frozen species whose |P| or |L*y| exceeds RCNTRL(12) re-enters the solve
 * as the last row of the compressed pattern, with the columns active at that
 * moment; ORD records the order of entry (-1 frozen, 0 active from the
 * start, t the t-th appended species). */
typedef struct {
  unsigned char DO_SLV[NVAR];
  int ORD[NVAR], nappend;
  int SPC_MAP[NVAR], iSPC_MAP[NVAR];
  int rNVAR, cNONZERO;
  int JVS_MAP[LU_NONZERO], cLU_IROW[LU_NONZERO], cLU_ICOL[LU_NONZERO];
  int cLU_CROW[NVAR + 1], cLU_DIAG[NVAR + 1];
} ar_map_t;

/* the reduction set-up of ros_yIntegrator (:917-1000), 0-based; keep[i]
 * marks species kept active (keepSpcActive) when keep is not NULL */
static void ar_build(ar_map_t* R, const double* Prod, const double* LossY, double AR_thr,
                     const unsigned char* keep) {
  int NRMV = 0, S = 0;
  for (int i = 0; i < NVAR; ++i) {
    R->DO_SLV[i] = 1;
    R->ORD[i] = 0;
    R->iSPC_MAP[i] = -1;
  }
  R->nappend = 0;
  for (int i = 0; i < NVAR; ++i) {
    if ((!keep || !keep[i]) && fabs(LossY[i]) < AR_thr && fabs(Prod[i]) < AR_thr) {
      NRMV = NRMV + 1;
      R->DO_SLV[i] = 0;
      R->ORD[i] = -1;
      continue;
    }
    R->SPC_MAP[S] = i;
    R->iSPC_MAP[i] = S;
    S = S + 1;
  }
  R->rNVAR = NVAR - NRMV;
  int II = 0, III = 0, idx = 0, i = 0;
  for (; i < LU_NONZERO; ++i) { /* ScanFirstNonZero */
    if (R->DO_SLV[ORACLE_LU_IROW[i]] && R->DO_SLV[ORACLE_LU_ICOL[i]]) {
      idx = 1;
      R->cLU_IROW[0] = R->iSPC_MAP[ORACLE_LU_IROW[i]];
      R->cLU_ICOL[0] = R->iSPC_MAP[ORACLE_LU_ICOL[i]];
      R->JVS_MAP[0] = i;
      break;
    }
  }
  for (i = i + 1; i < LU_NONZERO; ++i) {
    if (R->DO_SLV[ORACLE_LU_IROW[i]] && R->DO_SLV[ORACLE_LU_ICOL[i]]) {
      idx = idx + 1;
      R->cLU_IROW[idx - 1] = R->iSPC_MAP[ORACLE_LU_IROW[i]];
      R->cLU_ICOL[idx - 1] = R->iSPC_MAP[ORACLE_LU_ICOL[i]];
      R->JVS_MAP[idx - 1] = i;
      if (R->cLU_IROW[idx - 1] != R->cLU_IROW[idx - 2]) {
        II = II + 1;
        R->cLU_CROW[II] = idx - 1;
      }
      if (R->cLU_IROW[idx - 1] == R->cLU_ICOL[idx - 1]) {
        III = III + 1;
        R->cLU_DIAG[III] = idx - 1;
      }
    }
  }
  R->cNONZERO = idx;
  R->cLU_CROW[0] = 0;
  R->cLU_DIAG[0] = 0;
  if (R->rNVAR > 0) {
    R->cLU_CROW[R->rNVAR] = R->cNONZERO;
    R->cLU_DIAG[R->rNVAR] = R->cLU_DIAG[R->rNVAR - 1] + 1;
  }
}

/* APPEND (:2663-2700), 0-based: species idx becomes the last row of the
 * compressed pattern, holding the entries of its row whose column is active
 * now; no other row gains column idx. */
static void ar_append(ar_map_t* R, int idx) {
  R->DO_SLV[idx] = 1;
  R->ORD[idx] = ++R->nappend;
  R->rNVAR = R->rNVAR + 1;
  const int r = R->rNVAR - 1;
  R->SPC_MAP[r] = idx;
  R->iSPC_MAP[idx] = r;
  for (int i = 0; i < LU_NONZERO; ++i) {
    if (ORACLE_LU_IROW[i] == idx && R->DO_SLV[ORACLE_LU_ICOL[i]]) {
      const int e = R->cNONZERO;
      R->cNONZERO = R->cNONZERO + 1;
      R->cLU_IROW[e] = R->iSPC_MAP[ORACLE_LU_IROW[i]];
      R->cLU_ICOL[e] = R->iSPC_MAP[ORACLE_LU_ICOL[i]];
      R->JVS_MAP[e] = i;
      if (e == 0 || R->cLU_IROW[e] != R->cLU_IROW[e - 1]) R->cLU_CROW[r] = e;
      if (R->cLU_IROW[e] == R->cLU_ICOL[e]) R->cLU_DIAG[r] = e;
    }
  }
  R->cLU_CROW[r + 1] = R->cNONZERO;
  R->cLU_DIAG[r + 1] = R->cLU_DIAG[r] + 1;
}

/* cKppDecomp (gckpp_Integrator.F90:2624-2661) on the compressed pattern */
static int ckpp_decomp(const ar_map_t* R, double* JVS) {
  double W[NVAR], a;
  for (int k = 0; k < R->rNVAR; ++k) {
    if (fabs(JVS[R->cLU_DIAG[k]]) < DBL_MIN) return k + 1;
    for (int kk = R->cLU_CROW[k]; kk < R->cLU_CROW[k + 1]; ++kk) W[R->cLU_ICOL[kk]] = JVS[kk];
    for (int kk = R->cLU_CROW[k]; kk < R->cLU_DIAG[k]; ++kk) {
      int j = R->cLU_ICOL[kk];
      a = -W[j] / JVS[R->cLU_DIAG[j]];
      W[j] = -a;
      for (int jj = R->cLU_DIAG[j] + 1; jj < R->cLU_CROW[j + 1]; ++jj) W[R->cLU_ICOL[jj]] = W[R->cLU_ICOL[jj]] + a * JVS[jj];
    }
    for (int kk = R->cLU_CROW[k]; kk < R->cLU_CROW[k + 1]; ++kk) JVS[kk] = W[R->cLU_ICOL[kk]];
  }
  return 0;
}

/* ros_cPrepareMatrix (:1773-1851) */
static void c_prepare_matrix(cellctx_t* cx, const ar_map_t* R, double* H, int Direction, double gam,
                             const double* Jac0, double* cGhimj, int* Singular) {
  int Nconsecutive = 0;
  *Singular = 1;
  while (*Singular) {
    for (int i = 0; i < R->cNONZERO; ++i) cGhimj[i] = -Jac0[R->JVS_MAP[i]];
    double ghinv = 1.0 / (Direction * (*H) * gam);
    for (int i = 0; i < R->rNVAR; ++i) cGhimj[R->cLU_DIAG[i]] = cGhimj[R->cLU_DIAG[i]] + ghinv;
    int ising = ckpp_decomp(R, cGhimj);
    cx->istatus[Ndec] += 1;
    if (ising == 0) {
      *Singular = 0;
    } else {
      cx->istatus[Nsng] += 1;
      Nconsecutive += 1;
      *Singular = 1;
      if (Nconsecutive <= 5) *H = (*H) * 0.5;
      else return;
    }
  }
}

/* The masked form of the same decomposition, for the GPU design: Jac0 with
 * every entry in a frozen row or column zeroed, so that Ghimj = -Jac0 +
 * ghinv I decouples the frozen species (a frozen row is ghinv on the
 * diagonal, 0 elsewhere), factored by the full KppDecomp.  Frozen entries
 * only ever contribute exact zeros, so the kept entries come out as
 * cKppDecomp leaves them.  An appended species' row keeps the columns that
 * entered no later than it, and its column is zeroed in the rows that
 * entered earlier: the compressed pattern with appended rows last, in the
 * original order (the eliminations of an appended row only reach rows that
 * precede it in both orders). */
static void masked_prepare_matrix(cellctx_t* cx, const ar_map_t* R, double* H, int Direction, double gam,
                                  const double* Jac0, double* Ghimj, int* Singular) {
  int Nconsecutive = 0;
  *Singular = 1;
  while (*Singular) {
    for (int i = 0; i < LU_NONZERO; ++i) {
      /* with appends: row r holds column c if c entered no later than r */
      const int orr = R->ORD[ORACLE_LU_IROW[i]], oc = R->ORD[ORACLE_LU_ICOL[i]];
      Ghimj[i] = -((orr >= 0 && oc >= 0 && oc <= orr) ? Jac0[i] : 0.0);
    }
    double ghinv = 1.0 / (Direction * (*H) * gam);
    for (int i = 0; i < NVAR; ++i) Ghimj[ORACLE_LU_DIAG[i]] = Ghimj[ORACLE_LU_DIAG[i]] + ghinv;
    int ising = oracle_kpp_decomp(Ghimj);
    cx->istatus[Ndec] += 1;
    if (ising == 0) {
      *Singular = 0;
    } else {
      cx->istatus[Nsng] += 1;
      Nconsecutive += 1;
      *Singular = 1;
      if (Nconsecutive <= 5) *H = (*H) * 0.5;
      else return;
    }
  }
}

static void ros_yintegrator(cellctx_t* cx, const method_t* m, double* Y, double Tstart, double Tend, double* Tout,
                            const double* AbsTol, const double* RelTol, int Autonomous, int VectorTol,
                            int Max_no_steps, double Roundoff, double Hmin, double Hmax, double Hstart,
                            double FacMin, double FacMax, double FacRej, double FacSafe, double threshold,
                            int AR_target_spc, double AR_thr_ratio, const unsigned char* keep, int masked,
                            int append, int* IERR) {
  double Ynew[NVAR], Fcn0[NVAR], Fcn[NVAR], Prod[NVAR], Loss[NVAR], LossY[NVAR], K[6 * NVAR], dFdT[NVAR];
  double Prd0[NVAR], Los0[NVAR];
  double Yerr[NVAR];
  static __thread double Jac0[LU_NONZERO], Ghimj[LU_NONZERO], cGhimj[LU_NONZERO];
  static __thread ar_map_t R;
  double H, Hnew, HC, HG, Fac, Err, alpha_factor, AR_thr;
  int Direction, ioffset, j, istage, RejectLastH, RejectMoreH, Singular, reduced = 0;
  const double DeltaMin = 1.0e-5;
  double T = Tstart;
  cx->rstatus[Nhexit] = 0.0;
  H = fmin(fmax(fabs(Hmin), fabs(Hstart)), fabs(Hmax));
  if (fabs(H) <= 10.0 * Roundoff) H = DeltaMin;
  Direction = (Tend >= Tstart) ? +1 : -1;
  H = Direction * H;
  RejectLastH = 0;
  RejectMoreH = 0;
  memset(K, 0, sizeof(K));
  memset(Ghimj, 0, sizeof(Ghimj));
  memset(dFdT, 0, sizeof(dFdT));
  memset(Prod, 0, sizeof(Prod));
  memset(Loss, 0, sizeof(Loss));

  while ((Direction > 0 && ((T - Tend) + Roundoff <= 0.0)) || (Direction < 0 && ((Tend - T) + Roundoff <= 0.0))) {
    if (cx->istatus[Nstp] > Max_no_steps) { *IERR = -6; *Tout = T; return; }
    if (((T + 0.1 * H) == T) || (H <= Roundoff)) { *IERR = -7; *Tout = T; return; }
    H = fmin(H, fabs(Tend - T));
    if (append || T == Tstart) { /* FunSplitF: production and loss as well (every step in ros_yIntegratorA) */
      oracle_fun_pd(Y, cx->fix, cx->rct, Prod, Loss);
      for (int i = 0; i < NVAR; ++i) {
        LossY[i] = Loss[i] * Y[i];
        Fcn0[i] = Prod[i] - LossY[i];
      }
    } else {
      fun_template(cx, Y, Fcn0);
    }
    cx->istatus[Nfun] += 1;
    if (!reduced) {
      AR_thr = threshold;
      if (AR_target_spc > 0) {
        AR_thr = AR_thr_ratio * fmax(LossY[AR_target_spc - 1], Prod[AR_target_spc - 1]);
        cx->rstatus[3] = AR_thr; /* RSTATUS(NARthr) */
      }
      ar_build(&R, Prod, LossY, AR_thr, keep);
      memcpy(Prd0, Prod, sizeof(Prd0)); /* for AutoReduce_1stOrder */
      memcpy(Los0, Loss, sizeof(Los0));
      reduced = 1;
    }
    if (append) /* :1460-1474, against RCNTRL(12) itself, in species order */
      for (int i = 0; i < NVAR; ++i)
        if (!R.DO_SLV[i] && (fabs(LossY[i]) > threshold || fabs(Prod[i]) > threshold)) ar_append(&R, i);
    if (!Autonomous) fun_time_derivative(cx, T, Roundoff, Y, Fcn0, dFdT);
    jac_template(cx, Y, Jac0);
    cx->istatus[Njac] += 1;
    for (;;) { /* UntilAccepted */
      if (masked) {
        masked_prepare_matrix(cx, &R, &H, Direction, m->Gamma[0], Jac0, Ghimj, &Singular);
      } else {
        c_prepare_matrix(cx, &R, &H, Direction, m->Gamma[0], Jac0, cGhimj, &Singular);
      }
      if (Singular) { *IERR = -8; *Tout = T; return; }
      if (!masked)
        for (int i = 0; i < R.cNONZERO; ++i) Ghimj[R.JVS_MAP[i]] = cGhimj[i];
      for (istage = 1; istage <= m->S; ++istage) {
        ioffset = NVAR * (istage - 1);
        if (istage == 1) {
          memcpy(Fcn, Fcn0, sizeof(Fcn));
        } else if (m->NewF[istage - 1]) {
          memcpy(Ynew, Y, sizeof(Ynew));
          for (j = 1; j <= istage - 1; ++j) {
            alpha_factor = m->A[(istage - 1) * (istage - 2) / 2 + j - 1];
            for (int i = 0; i < R.rNVAR; ++i)
              Ynew[R.SPC_MAP[i]] = Ynew[R.SPC_MAP[i]] + alpha_factor * K[NVAR * (j - 1) + R.SPC_MAP[i]];
          }
          fun_template(cx, Ynew, Fcn);
          cx->istatus[Nfun] += 1;
        }
        if (istage > 1) {
          HC = m->C[(istage - 1) * (istage - 2) / 2] / (Direction * H);
          for (int i = 0; i < R.rNVAR; ++i) K[ioffset + R.SPC_MAP[i]] = Fcn[R.SPC_MAP[i]] + HC * K[R.SPC_MAP[i]];
        }
        if (istage == 1)
          for (int i = 0; i < R.rNVAR; ++i) K[ioffset + R.SPC_MAP[i]] = Fcn[R.SPC_MAP[i]];
        for (j = 2; j <= istage - 1; ++j) {
          HC = m->C[(istage - 1) * (istage - 2) / 2 + j - 1] / (Direction * H);
          for (int i = 0; i < R.rNVAR; ++i)
            K[ioffset + R.SPC_MAP[i]] = K[ioffset + R.SPC_MAP[i]] + HC * K[NVAR * (j - 1) + R.SPC_MAP[i]];
        }
        if (!Autonomous && m->Gamma[istage - 1] != 0.0) {
          HG = Direction * H * m->Gamma[istage - 1];
          for (int i = 0; i < R.rNVAR; ++i)
            K[ioffset + R.SPC_MAP[i]] = K[ioffset + R.SPC_MAP[i]] + HG * dFdT[R.SPC_MAP[i]];
        }
        if (masked) /* frozen right-hand sides are 0, the full KppSolve keeps them 0 */
          oracle_kpp_solve(Ghimj, K + ioffset);
        else
          oracle_kpp_solve_slv(Ghimj, K + ioffset, R.DO_SLV);
        cx->istatus[Nsol] += 1;
      }
      memcpy(Ynew, Y, sizeof(Ynew));
      memset(Yerr, 0, sizeof(Yerr));
      for (j = 1; j <= m->S; ++j)
        for (int i = 0; i < R.rNVAR; ++i) {
          Ynew[R.SPC_MAP[i]] = Ynew[R.SPC_MAP[i]] + m->M[j - 1] * K[NVAR * (j - 1) + R.SPC_MAP[i]];
          Yerr[R.SPC_MAP[i]] = Yerr[R.SPC_MAP[i]] + m->E[j - 1] * K[NVAR * (j - 1) + R.SPC_MAP[i]];
        }
      Err = error_norm(Y, Ynew, Yerr, AbsTol, RelTol, VectorTol);
      Fac = fmin(FacMax, fmax(FacMin, FacSafe / pow(Err, 1.0 / m->ELO)));
      Hnew = H * Fac;
      cx->istatus[Nstp] += 1;
      if ((Err <= 1.0) || (H <= Hmin)) {
        cx->istatus[Nacc] += 1;
        memcpy(Y, Ynew, sizeof(Ynew));
        T = T + Direction * H;
        Hnew = fmax(Hmin, fmin(Hnew, Hmax));
        if (RejectLastH) Hnew = fmin(Hnew, H);
        cx->rstatus[Nhexit] = H;
        cx->rstatus[Nhnew] = Hnew;
        cx->rstatus[Ntexit] = T;
        RejectLastH = 0;
        RejectMoreH = 0;
        H = Hnew;
        break;
      } else {
        if (RejectMoreH) Hnew = H * FacRej;
        RejectMoreH = RejectLastH;
        RejectLastH = 1;
        H = Hnew;
        if (cx->istatus[Nacc] >= 1) cx->istatus[Nrej] += 1;
      }
    }
  }
  /* AutoReduce_1stOrder (:1702-1712) for the frozen species */
  for (int i = 0; i < NVAR; ++i) {
    if (!R.DO_SLV[i]) {
      const double k = Los0[i];
      if (k <= 1.0e-30) continue;
      if (Y[i] <= 1.0e-30) continue;
      const double term = Prd0[i] / k;
      Y[i] = term + (Y[i] - term) * exp(-k * (Tend - Tstart));
    }
  }
  *Tout = T;
  *IERR = 1;
}

/* keepActive and keepSpcActive (gckpp_Global; fullchem_mod.F90:510-515 and
 * :585-587 set them through fullchem_AutoReduceFuncs.F90:47-110, 128-140):
 * species of the mask are never frozen by the reduction.  Off by default. */
static unsigned char g_keep[NVAR];
static int g_keep_on = 0;

void oracle_set_keep(const unsigned char* keep) {
  g_keep_on = keep != 0;
  for (int i = 0; i < NVAR; ++i) g_keep[i] = keep ? (keep[i] != 0) : 0;
}

void oracle_integrate(double* C, const double* RCONST, const double* atol, const double* rtol, double tin,
                      double tout, const int* icntrl_u, const double* rcntrl_u, int* istatus_u, double* rstatus_u,
                      int* ierr_u) {
  int ICNTRL[20];
  double RCNTRL[20];
  cellctx_t cx;
  memset(ICNTRL, 0, sizeof(ICNTRL));
  memset(RCNTRL, 0, sizeof(RCNTRL));
  memset(&cx, 0, sizeof(cx));
  ICNTRL[14] = 5;
  if (icntrl_u)
    for (int i = 0; i < 20; ++i) if (icntrl_u[i] != 0) ICNTRL[i] = icntrl_u[i];
  if (rcntrl_u)
    for (int i = 0; i < 20; ++i) if (rcntrl_u[i] > 0) RCNTRL[i] = rcntrl_u[i];
  cx.fix = C + NVAR;
  cx.rct = RCONST;
  int IERR = 0;
  /* Rosenbrock setup */
  method_t m;
  int Autonomous = !(ICNTRL[0] == 0);
  int VectorTol = (ICNTRL[1] == 0);
  int UplimTol = VectorTol ? NVAR : 1;
  int Max_no_steps = 200000;
  double Roundoff = wlamch_e();
  double Hmin, Hmax, Hstart, FacMin, FacMax, FacRej, FacSafe;
  if (!method_init(ICNTRL[2], &m)) { IERR = -2; goto done; }
  if (ICNTRL[3] == 0) Max_no_steps = 200000;
  else if (ICNTRL[3] > 0) Max_no_steps = ICNTRL[3];
  else { IERR = -1; goto done; }
  if (RCNTRL[0] == 0.0) Hmin = 0.0;
  else if (RCNTRL[0] > 0.0) Hmin = RCNTRL[0];
  else { IERR = -3; goto done; }
  if (RCNTRL[1] == 0.0) Hmax = fabs(tout - tin);
  else if (RCNTRL[1] > 0.0) Hmax = fmin(fabs(RCNTRL[1]), fabs(tout - tin));
  else { IERR = -3; goto done; }
  if (RCNTRL[2] == 0.0) Hstart = fmax(Hmin, 1.0e-5);
  else if (RCNTRL[2] > 0.0) Hstart = fmin(fabs(RCNTRL[2]), fabs(tout - tin));
  else { IERR = -3; goto done; }
  FacMin = RCNTRL[3] == 0.0 ? 0.2 : RCNTRL[3];
  FacMax = RCNTRL[4] == 0.0 ? 6.0 : RCNTRL[4];
  FacRej = RCNTRL[5] == 0.0 ? 0.1 : RCNTRL[5];
  FacSafe = RCNTRL[6] == 0.0 ? 0.9 : RCNTRL[6];
  for (int i = 0; i < UplimTol; ++i)
    if ((atol[i] <= 0.0) || (rtol[i] <= 10.0 * Roundoff) || (rtol[i] >= 1.0)) { IERR = -5; goto done; }
  {
    double Texit;
    /* auto-reduction (gckpp_Integrator.F90:388-394, 478-520): ICNTRL(12) = 1
     * selects ros_yIntegrator with threshold RCNTRL(12) (default 100) or, with
     * ICNTRL(14) = target species, RCNTRL(14) x max(P, L*y) of that species;
     * keepActive with the mask of oracle_set_keep; ICNTRL(13) = 1 selects
     * the append form, ros_yIntegratorA.  ICNTRL(20) = 7 (unused by the reference)
     * selects the masked-full decomposition of the GPU design instead of the
     * compressed one (tests only). */
    const int Autoreduce = ICNTRL[11] == 1;
    if (Autoreduce) {
      const double threshold = RCNTRL[11] > 0.0 ? RCNTRL[11] : 1.0e2;
      ros_yintegrator(&cx, &m, C, tin, tout, &Texit, atol, rtol, Autonomous, VectorTol, Max_no_steps, Roundoff,
                      Hmin, Hmax, Hstart, FacMin, FacMax, FacRej, FacSafe, threshold, ICNTRL[13], RCNTRL[13],
                      g_keep_on ? g_keep : 0, ICNTRL[19] == 7, ICNTRL[12] == 1, &IERR);
    } else {
      ros_integrator(&cx, &m, C, tin, tout, &Texit, atol, rtol, Autonomous, VectorTol, Max_no_steps, Roundoff,
                     Hmin, Hmax, Hstart, FacMin, FacMax, FacRej, FacSafe, ICNTRL[15] == 1, &IERR);
    }
  }
done:
  if (istatus_u) memcpy(istatus_u, cx.istatus, sizeof(cx.istatus));
  if (rstatus_u) memcpy(rstatus_u, cx.rstatus, sizeof(cx.rstatus));
  if (ierr_u) *ierr_u = IERR;
}

int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* The batch over cells; ar_thr/ar_target/ar_ratio, when given, are each
 * cell's RCNTRL(12), ICNTRL(14) and RCNTRL(14) (fullchem_AutoReduceFuncs.F90:
 * 293-343 sets them per grid box). */
void oracle_integrate_batch_ar(int ncell, double tin, double tout, double* c, long long ldc, const double* rconst,
                               long long ldr, const double* atol, const double* rtol, const int* icntrl_u,
                               const double* rcntrl_u, const double* hstart, int* istatus, double* rstatus,
                               long long ldo, int* ierr, int nthreads, const double* ar_thr, const int* ar_target,
                               const double* ar_ratio) {
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 24) num_threads(nthreads)
#endif
  for (int cell = 0; cell < ncell; ++cell) {
    double C[NSPEC], R[NREACT], rc[20], rs[20];
    int is[20], ie;
    for (int k = 0; k < NSPEC; ++k) C[k] = c[(long long)k * ldc + cell];
    for (int k = 0; k < NREACT; ++k) R[k] = rconst[(long long)k * ldr + cell];
    int ic[20];
    for (int k = 0; k < 20; ++k) rc[k] = rcntrl_u ? rcntrl_u[k] : 0.0;
    for (int k = 0; k < 20; ++k) ic[k] = icntrl_u ? icntrl_u[k] : 0;
    if (hstart) rc[2] = hstart[cell];
    if (ar_thr) rc[11] = ar_thr[cell];
    if (ar_target) ic[13] = ar_target[cell];
    if (ar_ratio) rc[13] = ar_ratio[cell];
    oracle_integrate(C, R, atol, rtol, tin, tout, ic, rc, is, rs, &ie);
    for (int k = 0; k < NVAR; ++k) c[(long long)k * ldc + cell] = C[k];
    if (istatus) for (int k = 0; k < 20; ++k) istatus[(long long)k * ldo + cell] = is[k];
    if (rstatus) for (int k = 0; k < 20; ++k) rstatus[(long long)k * ldo + cell] = rs[k];
    ierr[cell] = ie;
  }
  (void)nthreads;
}

void oracle_integrate_batch(int ncell, double tin, double tout, double* c, long long ldc, const double* rconst,
                            long long ldr, const double* atol, const double* rtol, const int* icntrl_u,
                            const double* rcntrl_u, const double* hstart, int* istatus, double* rstatus,
                            long long ldo, int* ierr, int nthreads) {
  oracle_integrate_batch_ar(ncell, tin, tout, c, ldc, rconst, ldr, atol, rtol, icntrl_u, rcntrl_u, hstart, istatus,
                            rstatus, ldo, ierr, nthreads, 0, 0, 0);
}

void oracle_update_rconst_het_batch(int ncell, const double* met, long long ldm, const double* photol,
                                    long long ldp, const double* c, long long ldc, const double* het, long long ldh,
                                    double* rconst, long long ldr) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int cell = 0; cell < ncell; ++cell) {
    double M[18], P[200], C[NSPEC], R[NREACT];
    for (int k = 0; k < 18; ++k) M[k] = met[(long long)k * ldm + cell];
    for (int k = 0; k < 200; ++k) P[k] = photol[(long long)k * ldp + cell];
    for (int k = 0; k < NSPEC; ++k) C[k] = c[(long long)k * ldc + cell];
    oracle_update_rconst_het(M, P, C, het ? het + cell : 0, ldh, R);
    for (int k = 0; k < NREACT; ++k) rconst[(long long)k * ldr + cell] = R[k];
  }
}

void oracle_update_rconst_batch(int ncell, const double* met, long long ldm, const double* photol, long long ldp,
                                const double* c, long long ldc, double* rconst, long long ldr) {
  oracle_update_rconst_het_batch(ncell, met, ldm, photol, ldp, c, ldc, 0, 0, rconst, ldr);
}
