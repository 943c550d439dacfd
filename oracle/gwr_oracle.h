/*
 * gwr_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of libgwmodel's GWRBasic hot path (GWRBasic::fit with
 * golden-section bandwidth selection), used by tests/, by the smoke check
 * and by bench.py's CPU-baseline leg as the parity checker.  Nothing in the
 * product library links or calls it.
 *
 * Pinned against the known answers of the reference's own tests
 * (test/testGWRBasic.cpp:40-137, 186-240) on the londonhp100 fixture; see
 * tests/test_oracle_golden.py.
 *
 * Matrices are column-major (Armadillo layout): element (i, k) of an
 * n x p matrix is at [i + k*n].
 */
#ifndef GWR_ORACLE_H
#define GWR_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_AIC 0 /* GWRBasic::BandwidthSelectionCriterionType::AIC */
#define ORC_CV 1  /* GWRBasic::BandwidthSelectionCriterionType::CV */


typedef struct orc_problem
{
    int n, p;
    const double* x;      /* n x p */
    const double* y;      /* n */
    const double* coords; /* n x 2: column 0 = x or longitude, column 1 = y or latitude */
    int geographic;       /* CRSDistance(isGeographic) */
    int threads;          /* OpenMP threads (mOmpThreadNum) */
} orc_problem;

/* CRSDistance::SpGcdist with libm (CRSDistance.cpp:15-69). */
double orc_gcdist_libm(double lon1, double lon2, double lat1, double lat2);

/* CRSDistance::distance(focus) for focus points == data points (CRSDistance.cpp:122-131). */
void orc_distance_row(const orc_problem* pb, int focus, double* out);
/* CRSDistance::maxDistance (CRSDistance.cpp:133-143). */
double orc_max_distance(const orc_problem* pb);

/* BandwidthWeight::weight (BandwidthWeight.cpp:35-61).  Returns 0, or -1 when
 * the adaptive bandwidth indexes outside the sorted distances. */
int orc_weight(const double* dist, int n, double bw, int adaptive, int kernel, double* w);

/* Adaptive threshold alone: the fixbw of BandwidthWeight.cpp:40-53. */
int orc_adaptive_threshold(const double* dist, int n, double bw, double* fixbw);

/* bandwidthSizeCriterion{AIC,CV}Omp (GWRBasic.cpp:440-535).  Returns the
 * criterion, DBL_MAX when a local system is not SPD or the value is not
 * finite.  shat_out (may be NULL) receives (trS, trStS) for AIC. */
double orc_criterion(const orc_problem* pb, double bw, int adaptive, int kernel, int criterion,
                     double* shat_out);

/* The same criterion restricted to rows [row0, row1) and summed: the timed
 * CPU-baseline sample.  Returns the partial sum of s_ii (AIC) or the CV sum. */
double orc_criterion_rows(const orc_problem* pb, double bw, int adaptive, int kernel, int criterion,
                          int row0, int row1);

/* indepVarsSelectionCriterionOmp (GWRBasic.cpp:537-580): AICc with w == 1 on
 * the columns cols[0..ncols). */
double orc_indep_vars_criterion(const orc_problem* pb, const int* cols, int ncols);

/* fitOmp (GWRBasic.cpp:386-438).  betas and betas_se are n x p; shat has 2
 * entries; qdiag n; S is n x n when store_s, else 1 x n (the last row).
 * Returns 0, or -1 when a local system is not SPD. */
int orc_fit_core(const orc_problem* pb, double bw, int adaptive, int kernel, int store_s,
                 double* betas, double* betas_se, double* shat, double* qdiag, double* S);

/* BandwidthSelector::optimize (BandwidthSelector.cpp:6-81) over orc_criterion.
 * Writes the chosen bandwidth; list_bw/list_f (capacity cap) receive the
 * (bandwidth, criterion) pairs sorted by bandwidth (:83-95).  Returns the
 * number of pairs, or -1 for "Invalid initial values." */
/* GWRBasic::predictSerial: betas (nr x p column-major) at nr locations (nr x 2 column-major). */
int orc_predict(const orc_problem* pb, int nr, const double* loc, double bw, int adaptive, int kernel,
                double* betas);

int orc_golden(const orc_problem* pb, double bw0, int adaptive, int kernel, int criterion,
               double lower, double upper, double* bw_out, double* list_bw, double* list_f, int cap);

/* GWRBasic::CalcDiagnostic (GWRBasic.cpp:21-34): out = RSS, AIC, AICc, ENP,
 * EDF, R2, R2adj. */
void orc_diagnostic(const orc_problem* pb, const double* betas, const double* shat, double* out);

/* Local Cholesky inverse of an SPD p x p matrix in place (inv_sympd); 0 or -1. */
int orc_inv_sympd(double* a, int p);

/* GWRMultiscale::fit (serial forms). */
#define ORC_MGWR_INIT_NULL 0
#define ORC_MGWR_INIT_INITIAL 1
#define ORC_MGWR_INIT_SPECIFIED 2
#define ORC_MGWR_CV 0
#define ORC_MGWR_AIC 1
#define ORC_MGWR_CVR 0
#define ORC_MGWR_DCVR 1
typedef struct orc_mgwr_opts
{
    const int* adaptive;           /* per variable */
    const int* kernel;
    const double* bw0;             /* initial bandwidths */
    const int* init_type;          /* ORC_MGWR_INIT_* */
    const int* approach;           /* ORC_MGWR_CV / ORC_MGWR_AIC */
    const int* centered;
    const double* select_threshold;
    int retry_times, max_iteration, criterion_type;
    double criterion_threshold;
    int adaptive_lower;
    int has_lower, has_upper;
    double lower, upper;
    int has_hat_matrix, has_intercept;
} orc_mgwr_opts;
typedef struct orc_mgwr_out
{
    double* betas;     /* n x p */
    double* betas_se;  /* n x p (hat matrix only) */
    double* bws;       /* p */
    double init_bw;
    double shat[2];
    double rss;
    double diag[6];    /* RSS, AICc, ENP, EDF, R2, adjusted R2 */
    int iterations;
} orc_mgwr_out;
int orc_mgwr_fit(const orc_problem* pb, const orc_mgwr_opts* o, orc_mgwr_out* out);

#ifdef __cplusplus
}
#endif
#endif /* GWR_ORACLE_H */
