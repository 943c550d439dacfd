/*
 * gwr_oracle.c -- TEST INFRASTRUCTURE ONLY: the CPU oracle for the GWRBasic
 * hot path.  Every function restates the reference line range it cites
 * (paths inside libgwmodel).  Build with -ffp-contract=off so that distances
 * and weights round exactly as the reference's expressions do.  Nothing of
 * the engine is compiled in: distances, kernels and the great-circle formula
 * (with the platform libm) are restated here from the reference alone.
 */
#include "gwr_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* DOUBLE_EPS compile definition of the reference (src/CMakeLists.txt:33-36). */
#define ORC_DOUBLE_EPS 1e-8

#define X_(pb, i, k) ((pb)->x[(size_t)(i) + (size_t)(k) * (size_t)(pb)->n])
#define U_(pb, i) ((pb)->coords[(size_t)(i)])
#define V_(pb, i) ((pb)->coords[(size_t)(i) + (size_t)(pb)->n])

static int orc_threads(const orc_problem* pb)
{
    return pb->threads > 0 ? pb->threads : 1;
}

static int orc_thread_id(void)
{
#ifdef _OPENMP
    return omp_get_thread_num();
#else
    return 0;
#endif
}

/* ---------------------------------------------------------------- distance */

/* CRSDistance::SpGcdist (CRSDistance.cpp:15-69) with libm, line for line. */
double orc_gcdist_libm(double lon1, double lon2, double lat1, double lat2)
{
    double F, G, L, sinG2, cosG2, sinF2, cosF2, sinL2, cosL2, S, C;
    double w, R, a, f, D, H1, H2;
    double lat1R, lat2R, lon1R, lon2R, DE2RA;
    DE2RA = M_PI / 180;
    a = 6378.137;
    f = 1.0 / 298.257223563;
    if (fabs(lat1 - lat2) < ORC_DOUBLE_EPS)
    {
        if (fabs(lon1 - lon2) < ORC_DOUBLE_EPS)
            return 0.0;
        else if (fabs((fabs(lon1) + fabs(lon2)) - 360.0) < ORC_DOUBLE_EPS)
            return 0.0;
    }
    lat1R = lat1 * DE2RA;
    lat2R = lat2 * DE2RA;
    lon1R = lon1 * DE2RA;
    lon2R = lon2 * DE2RA;
    F = (lat1R + lat2R) / 2.0;
    G = (lat1R - lat2R) / 2.0;
    L = (lon1R - lon2R) / 2.0;
    sinG2 = pow(sin(G), 2);
    cosG2 = pow(cos(G), 2);
    sinF2 = pow(sin(F), 2);
    cosF2 = pow(cos(F), 2);
    sinL2 = pow(sin(L), 2);
    cosL2 = pow(cos(L), 2);
    S = sinG2 * cosL2 + cosF2 * sinL2;
    C = cosG2 * cosL2 + sinF2 * sinL2;
    w = atan(sqrt(S / C));
    R = sqrt(S * C) / w;
    D = 2 * w * a;
    H1 = (3 * R - 1) / (2 * C);
    H2 = (3 * R + 1) / (2 * S);
    return D * (1 + f * H1 * sinF2 * cosG2 - f * H2 * cosF2 * sinG2);
}

/* CRSDistance::EuclideanDistance (CRSDistance.h:95-99): diff = data - focus,
 * sqrt(sum(diff % diff, 1)). */
static double orc_planar_dist(double ud, double vd, double uf, double vf)
{
    double dx = ud - uf, dy = vd - vf;
    return sqrt(dx * dx + dy * dy);
}

/* The five kernel functions (BandwidthWeight.h:68-121) for one element: the
 * indicator (dist < bw) multiplies the polynomial as a 0/1 double. */
static double orc_kernel_weight(int kernel, double d, double bw)
{
    switch (kernel)
    {
    case 0: /* Gaussian */
        return exp((d * d) / ((-2.0) * (bw * bw)));
    case 1: /* Exponential */
        return exp(-d / bw);
    case 2: /* Bisquare */
    {
        double t = 1.0 - (d * d) / (bw * bw);
        return (d < bw ? 1.0 : 0.0) * (t * t);
    }
    case 3: /* Tricube */
    {
        double t = 1.0 - (d * d * d) / (bw * bw * bw);
        return (d < bw ? 1.0 : 0.0) * (t * t * t);
    }
    default: /* Boxcar */
        return (d < bw ? 1.0 : 0.0) * 1.0;
    }
}

/* CRSDistance::distance(focus) (CRSDistance.cpp:122-131) with focus points ==
 * data points; planar EuclideanDistance (CRSDistance.h:95-99) or
 * SpatialDistance (CRSDistance.cpp:71-81: SpGcdist(data lon, focus lon,
 * data lat, focus lat)). */
void orc_distance_row(const orc_problem* pb, int focus, double* out)
{
    const double uf = U_(pb, focus), vf = V_(pb, focus);
    for (int j = 0; j < pb->n; j++)
    {
        if (!pb->geographic)
            out[j] = orc_planar_dist(U_(pb, j), V_(pb, j), uf, vf);
        else
            out[j] = orc_gcdist_libm(U_(pb, j), uf, V_(pb, j), vf);
    }
}

/* CRSDistance::maxDistance (CRSDistance.cpp:133-143). */
double orc_max_distance(const orc_problem* pb)
{
    const int n = pb->n, T = orc_threads(pb);
    double maxD = 0.0;
    double* buf = (double*)malloc(sizeof(double) * (size_t)n * (size_t)T);
#pragma omp parallel for num_threads(T) schedule(dynamic, 16) reduction(max : maxD)
    for (int i = 0; i < n; i++)
    {
        double* d = buf + (size_t)n * (size_t)orc_thread_id();
        orc_distance_row(pb, i, d);
        double m = d[0];
        for (int j = 1; j < n; j++)
            if (d[j] > m) m = d[j];
        maxD = m > maxD ? m : maxD;
    }
    free(buf);
    return maxD;
}

/* ------------------------------------------------------------------ weight */

static int cmp_double(const void* a, const void* b)
{
    double x = *(const double*)a, y = *(const double*)b;
    return (x > y) - (x < y);
}

/* fixbw of the adaptive branch, BandwidthWeight.cpp:40-53. */
int orc_adaptive_threshold(const double* dist, int n, double bw, double* fixbw)
{
    double dn = bw / n;
    if (dn < 1)
    {
        double b0 = floor(bw), bx = bw - b0;
        long long i0 = (long long)(int)b0 - 1, i1 = (long long)(int)b0;
        if (i0 < 0 || i1 >= n) return -1; /* Armadillo bounds error */
        double* s = (double*)malloc(sizeof(double) * (size_t)n);
        memcpy(s, dist, sizeof(double) * (size_t)n);
        qsort(s, (size_t)n, sizeof(double), cmp_double);
        double d0 = s[i0], d1 = s[i1];
        *fixbw = d0 + (d1 - d0) * bx;
        free(s);
    }
    else
    {
        double m = dist[0];
        for (int j = 1; j < n; j++)
            if (dist[j] > m) m = dist[j];
        *fixbw = dn * m;
    }
    return 0;
}

/* BandwidthWeight::weight (BandwidthWeight.cpp:35-61). */
int orc_weight(const double* dist, int n, double bw, int adaptive, int kernel, double* w)
{
    double b = bw;
    if (adaptive && orc_adaptive_threshold(dist, n, bw, &b) != 0) return -1;
    for (int j = 0; j < n; j++)
        w[j] = orc_kernel_weight(kernel, dist[j], b);
    return 0;
}

/* ------------------------------------------------------------ local solve */

/* inv_sympd: Cholesky A = L L^T (dpotrf), then A^-1 = L^-T L^-1 (dpotri).
 * Fails like dpotrf when a leading minor is not positive. */
int orc_inv_sympd(double* a, int p)
{
    /* factor in place, lower triangle, column-major a[i + j*p] */
    for (int j = 0; j < p; j++)
    {
        double s = a[j + j * p];
        for (int k = 0; k < j; k++)
            s -= a[j + k * p] * a[j + k * p];
        if (!(s > 0.0)) return -1;
        double ljj = sqrt(s);
        a[j + j * p] = ljj;
        for (int i = j + 1; i < p; i++)
        {
            double t = a[i + j * p];
            for (int k = 0; k < j; k++)
                t -= a[i + k * p] * a[j + k * p];
            a[i + j * p] = t / ljj;
        }
    }
    /* invert L in place (lower) */
    for (int j = 0; j < p; j++)
    {
        a[j + j * p] = 1.0 / a[j + j * p];
        for (int i = j + 1; i < p; i++)
        {
            double t = 0.0;
            for (int k = j; k < i; k++)
                t -= a[i + k * p] * a[k + j * p];
            a[i + j * p] = t / a[i + i * p];
        }
    }
    /* A^-1 = L^-T L^-1, fill both triangles */
    for (int j = 0; j < p; j++)
        for (int i = j; i < p; i++)
        {
            double t = 0.0;
            for (int k = i; k < p; k++)
                t += a[k + i * p] * a[k + j * p];
            a[i + j * p] = t; /* lower part now holds (i >= j) */
        }
    for (int j = 0; j < p; j++)
        for (int i = 0; i < j; i++)
            a[i + j * p] = a[j + i * p];
    return 0;
}

/* Per-thread scratch for one local regression. */
typedef struct
{
    double *d, *w, *xtw, *ci, *si, *a, *b, *beta;
} orc_ws;

static void ws_alloc(orc_ws* ws, int n, int p, int need_c)
{
    ws->d = (double*)malloc(sizeof(double) * (size_t)n);
    ws->w = (double*)malloc(sizeof(double) * (size_t)n);
    ws->xtw = (double*)malloc(sizeof(double) * (size_t)n * (size_t)p);
    ws->ci = need_c ? (double*)malloc(sizeof(double) * (size_t)n * (size_t)p) : NULL;
    ws->si = need_c ? (double*)malloc(sizeof(double) * (size_t)n) : NULL;
    ws->a = (double*)malloc(sizeof(double) * (size_t)p * (size_t)p);
    ws->b = (double*)malloc(sizeof(double) * (size_t)p);
    ws->beta = (double*)malloc(sizeof(double) * (size_t)p);
}

static void ws_free(orc_ws* ws)
{
    free(ws->d); free(ws->w); free(ws->xtw); free(ws->ci); free(ws->si);
    free(ws->a); free(ws->b); free(ws->beta);
}

/* xtw = trans(x.each_col() % w) (p x n, column-major: xtw[k + j*p]);
 * xtwx = xtw * x; xtwy = xtw * y; then inv_sympd and beta = inv * xtwy
 * (GWRBasic.cpp:500-508).  Returns -1 when not SPD. */
static int local_solve(const orc_problem* pb, const double* x, int p, orc_ws* ws)
{
    const int n = pb->n;
    for (int j = 0; j < n; j++)
        for (int k = 0; k < p; k++)
            ws->xtw[k + (size_t)j * p] = x[(size_t)j + (size_t)k * n] * ws->w[j];
    for (int c = 0; c < p; c++)
        for (int r = 0; r < p; r++)
        {
            double s = 0.0;
            for (int j = 0; j < n; j++)
                s += ws->xtw[r + (size_t)j * p] * x[(size_t)j + (size_t)c * n];
            ws->a[r + c * p] = s;
        }
    for (int r = 0; r < p; r++)
    {
        double s = 0.0;
        for (int j = 0; j < n; j++)
            s += ws->xtw[r + (size_t)j * p] * pb->y[j];
        ws->b[r] = s;
    }
    if (orc_inv_sympd(ws->a, p) != 0) return -1;
    for (int r = 0; r < p; r++)
    {
        double s = 0.0;
        for (int c = 0; c < p; c++)
            s += ws->a[r + c * p] * ws->b[c];
        ws->beta[r] = s;
    }
    return 0;
}

/* ci = inv * xtw (p x n); si = x.row(i) * ci (1 x n) (GWRBasic.cpp:509-510). */
static void hat_row(const orc_problem* pb, const double* x, int p, int i, orc_ws* ws)
{
    const int n = pb->n;
    for (int j = 0; j < n; j++)
        for (int r = 0; r < p; r++)
        {
            double s = 0.0;
            for (int c = 0; c < p; c++)
                s += ws->a[r + c * p] * ws->xtw[c + (size_t)j * p];
            ws->ci[r + (size_t)j * p] = s;
        }
    for (int j = 0; j < n; j++)
    {
        double s = 0.0;
        for (int r = 0; r < p; r++)
            s += x[(size_t)i + (size_t)r * n] * ws->ci[r + (size_t)j * p];
        ws->si[j] = s;
    }
}

/* GWRBase::RSS and AICc (GWRBase.h:41-94): betas is n x p. */
static double rss_of(const orc_problem* pb, const double* x, int p, const double* betas)
{
    const int n = pb->n;
    double ss = 0.0;
    for (int i = 0; i < n; i++)
    {
        double fit = 0.0;
        for (int k = 0; k < p; k++)
            fit += betas[(size_t)i + (size_t)k * n] * x[(size_t)i + (size_t)k * n];
        double r = pb->y[i] - fit;
        ss += r * r;
    }
    return ss;
}

static double aicc_of(double n, double rss, double trS)
{
    return n * log(rss / n) + n * log(2 * M_PI) + n * ((n + trS) / (n - 2 - trS));
}

/* ---------------------------------------------------------------- criteria */

typedef struct
{
    double sum0, sum1; /* AIC: trS, trStS;  CV: sum of squares */
    int ok;
} crit_part;

static crit_part criterion_rows_impl(const orc_problem* pb, double bw, int adaptive, int kernel,
                                     int criterion, int row0, int row1, double* betas)
{
    const int n = pb->n, p = pb->p, T = orc_threads(pb);
    const int need_c = criterion == ORC_AIC;
    orc_ws* ws = (orc_ws*)malloc(sizeof(orc_ws) * (size_t)T);
    for (int t = 0; t < T; t++) ws_alloc(&ws[t], n, p, need_c);
    double s0 = 0.0, s1 = 0.0;
    int ok = 1;
#pragma omp parallel for num_threads(T) schedule(dynamic, 1) reduction(+ : s0, s1) reduction(&& : ok)
    for (int i = row0; i < row1; i++)
    {
        orc_ws* w = &ws[orc_thread_id()];
        orc_distance_row(pb, i, w->d);
        if (orc_weight(w->d, n, bw, adaptive, kernel, w->w) != 0) { ok = 0; continue; }
        if (criterion == ORC_CV) w->w[i] = 0.0; /* GWRBasic.cpp:455 */
        if (local_solve(pb, pb->x, p, w) != 0) { ok = 0; continue; }
        if (criterion == ORC_CV)
        {
            /* res = y(i) - x.row(i) * beta (GWRBasic.cpp:462-467) */
            double yhat = 0.0;
            for (int k = 0; k < p; k++) yhat += X_(pb, i, k) * w->beta[k];
            double res = pb->y[i] - yhat;
            if (isfinite(res)) s0 += res * res;
            else ok = 0;
        }
        else
        {
            if (betas)
                for (int k = 0; k < p; k++) betas[(size_t)i + (size_t)k * n] = w->beta[k];
            hat_row(pb, pb->x, p, i, w);
            double ss = 0.0;
            for (int j = 0; j < n; j++) ss += w->si[j] * w->si[j];
            s0 += w->si[i]; /* shat(0) += si(0, i) */
            s1 += ss;       /* shat(1) += det(si * si.t()) */
        }
    }
    for (int t = 0; t < T; t++) ws_free(&ws[t]);
    free(ws);
    crit_part r = {s0, s1, ok};
    return r;
}

/* bandwidthSizeCriterionCVOmp / AICOmp (GWRBasic.cpp:440-535). */
double orc_criterion(const orc_problem* pb, double bw, int adaptive, int kernel, int criterion,
                     double* shat_out)
{
    const int n = pb->n, p = pb->p;
    double* betas = criterion == ORC_AIC ? (double*)calloc((size_t)n * (size_t)p, sizeof(double)) : NULL;
    crit_part r = criterion_rows_impl(pb, bw, adaptive, kernel, criterion, 0, n, betas);
    double value = DBL_MAX;
    if (r.ok)
    {
        if (criterion == ORC_CV)
            value = isfinite(r.sum0) ? r.sum0 : DBL_MAX;
        else
        {
            double v = aicc_of((double)n, rss_of(pb, pb->x, p, betas), r.sum0);
            value = isfinite(v) ? v : DBL_MAX;
            if (shat_out) { shat_out[0] = r.sum0; shat_out[1] = r.sum1; }
        }
    }
    free(betas);
    return value;
}

double orc_criterion_rows(const orc_problem* pb, double bw, int adaptive, int kernel, int criterion,
                          int row0, int row1)
{
    crit_part r = criterion_rows_impl(pb, bw, adaptive, kernel, criterion, row0, row1, NULL);
    return r.ok ? r.sum0 : DBL_MAX;
}

/* indepVarsSelectionCriterionOmp (GWRBasic.cpp:537-580): the AICc of the
 * model on columns cols with every weight equal to one. */
double orc_indep_vars_criterion(const orc_problem* pb, const int* cols, int ncols)
{
    const int n = pb->n, T = orc_threads(pb);
    double* x = (double*)malloc(sizeof(double) * (size_t)n * (size_t)ncols);
    for (int k = 0; k < ncols; k++)
        memcpy(x + (size_t)k * n, pb->x + (size_t)cols[k] * n, sizeof(double) * (size_t)n);
    double* betas = (double*)calloc((size_t)n * (size_t)ncols, sizeof(double));
    orc_ws* ws = (orc_ws*)malloc(sizeof(orc_ws) * (size_t)T);
    for (int t = 0; t < T; t++) ws_alloc(&ws[t], n, ncols, 1);
    double s0 = 0.0;
    int ok = 1;
#pragma omp parallel for num_threads(T) schedule(dynamic, 4) reduction(+ : s0) reduction(&& : ok)
    for (int i = 0; i < n; i++)
    {
        orc_ws* w = &ws[orc_thread_id()];
        for (int j = 0; j < n; j++) w->w[j] = 1.0;
        if (local_solve(pb, x, ncols, w) != 0) { ok = 0; continue; }
        for (int k = 0; k < ncols; k++) betas[(size_t)i + (size_t)k * n] = w->beta[k];
        hat_row(pb, x, ncols, i, w);
        s0 += w->si[i];
    }
    double value = DBL_MAX;
    if (ok) value = aicc_of((double)n, rss_of(pb, x, ncols, betas), s0);
    for (int t = 0; t < T; t++) ws_free(&ws[t]);
    free(ws);
    free(betas);
    free(x);
    return value;
}

/* ---------------------------------------------------------------- final fit */

/* fitOmp (GWRBasic.cpp:386-438). */
int orc_fit_core(const orc_problem* pb, double bw, int adaptive, int kernel, int store_s,
                 double* betas, double* betas_se, double* shat, double* qdiag, double* S)
{
    const int n = pb->n, p = pb->p, T = orc_threads(pb);
    orc_ws* ws = (orc_ws*)malloc(sizeof(orc_ws) * (size_t)T);
    double* qall = (double*)calloc((size_t)n * (size_t)T, sizeof(double));
    for (int t = 0; t < T; t++) ws_alloc(&ws[t], n, p, 1);
    const size_t srows = store_s ? (size_t)n : 1;
    double s0 = 0.0, s1 = 0.0;
    int ok = 1;
#pragma omp parallel for num_threads(T) schedule(dynamic, 1) reduction(+ : s0, s1) reduction(&& : ok)
    for (int i = 0; i < n; i++)
    {
        const int t = orc_thread_id();
        orc_ws* w = &ws[t];
        orc_distance_row(pb, i, w->d);
        if (orc_weight(w->d, n, bw, adaptive, kernel, w->w) != 0) { ok = 0; continue; }
        if (local_solve(pb, pb->x, p, w) != 0) { ok = 0; continue; }
        for (int k = 0; k < p; k++) betas[(size_t)i + (size_t)k * n] = w->beta[k];
        hat_row(pb, pb->x, p, i, w);
        /* betasSE.col(i) = sum(ci % ci, 1) */
        for (int r = 0; r < p; r++)
        {
            double s = 0.0;
            for (int j = 0; j < n; j++) s += w->ci[r + (size_t)j * p] * w->ci[r + (size_t)j * p];
            betas_se[(size_t)i + (size_t)r * n] = s;
        }
        double ss = 0.0;
        for (int j = 0; j < n; j++) ss += w->si[j] * w->si[j];
        s0 += w->si[i];
        s1 += ss;
        /* p = -si.t(); p(i) += 1; qDiag += p % p */
        double* q = qall + (size_t)n * (size_t)t;
        for (int j = 0; j < n; j++)
        {
            double v = -w->si[j];
            if (j == i) v += 1.0;
            q[j] += v * v;
        }
        const size_t row = store_s ? (size_t)i : 0;
        if (store_s || i == n - 1)
            for (int j = 0; j < n; j++) S[row + (size_t)j * srows] = w->si[j];
    }
    for (int j = 0; j < n; j++)
    {
        double s = 0.0;
        for (int t = 0; t < T; t++) s += qall[(size_t)n * (size_t)t + (size_t)j];
        qdiag[j] = s;
    }
    shat[0] = s0;
    shat[1] = s1;
    for (int t = 0; t < T; t++) ws_free(&ws[t]);
    free(ws);
    free(qall);
    return ok ? 0 : -1;
}

/* GWRBasic::predictSerial (GWRBasic.cpp:165-191): beta at nr locations
   (nr x 2 column-major) from the weights of each location's distances to the
   data (CRSDistance with the prediction parameter {locations, coords},
   GWRBasic.cpp:157-163: data point first, location second, as in a fit). */
int orc_predict(const orc_problem* pb, int nr, const double* loc, double bw, int adaptive, int kernel,
                double* betas)
{
    const int n = pb->n, p = pb->p, T = orc_threads(pb);
    orc_ws* ws = (orc_ws*)malloc(sizeof(orc_ws) * (size_t)T);
    for (int t = 0; t < T; t++) ws_alloc(&ws[t], n, p, 0);
    int ok = 1;
#pragma omp parallel for num_threads(T) schedule(dynamic, 1) reduction(&& : ok)
    for (int r = 0; r < nr; r++)
    {
        orc_ws* w = &ws[orc_thread_id()];
        const double uf = loc[r], vf = loc[(size_t)nr + r];
        for (int j = 0; j < n; j++)
        {
            if (!pb->geographic)
                w->d[j] = orc_planar_dist(U_(pb, j), V_(pb, j), uf, vf);
            else
                w->d[j] = orc_gcdist_libm(U_(pb, j), uf, V_(pb, j), vf);
        }
        if (orc_weight(w->d, n, bw, adaptive, kernel, w->w) != 0) { ok = 0; continue; }
        if (local_solve(pb, pb->x, p, w) != 0) { ok = 0; continue; }
        for (int k = 0; k < p; k++) betas[(size_t)r + (size_t)k * nr] = w->beta[k];
    }
    for (int t = 0; t < T; t++) ws_free(&ws[t]);
    free(ws);
    return ok ? 0 : -1;
}

/* ------------------------------------------------------------ golden search */

typedef struct
{
    double* bw;
    double* f;
    int n, cap;
} crit_map;

/* mBandwidthCriterion[x] = f (std::map insert-or-assign). */
static void map_put(crit_map* m, double x, double f)
{
    for (int i = 0; i < m->n; i++)
        if (m->bw[i] == x) { m->f[i] = f; return; }
    if (m->n < m->cap) { m->bw[m->n] = x; m->f[m->n] = f; m->n++; }
}

/* BandwidthSelector::optimize (BandwidthSelector.cpp:6-81). */
int orc_golden(const orc_problem* pb, double bw0, int adaptive, int kernel, int criterion,
               double lower, double upper, double* bw_out, double* list_bw, double* list_f, int cap)
{
    crit_map m = {list_bw, list_f, 0, cap};
    double xU = upper, xL = lower;
    const double eps = 1e-4;
    const double R = (sqrt(5) - 1) / 2;
    int iter = 0;
    double d = R * (xU - xL);
    double x1 = adaptive ? floor(xL + d) : (xL + d);
    double x2 = adaptive ? round(xU - d) : (xU - d);
    double f1 = orc_criterion(pb, x1, adaptive, kernel, criterion, NULL);
    double f2 = orc_criterion(pb, x2, adaptive, kernel, criterion, NULL);
    if (f1 == DBL_MAX && f2 == DBL_MAX) return -1; /* "Invalid initial values." */
    if (f1 < DBL_MAX) map_put(&m, x1, f1);
    if (f2 < DBL_MAX) map_put(&m, x2, f2);
    double d1 = f2 - f1;
    double xopt = f1 < f2 ? x1 : x2;
    double ea = 100;
    while ((fabs(d) > eps) && (fabs(d1) > eps) && iter < ea)
    {
        d = R * d;
        if (f1 < f2)
        {
            xL = x2;
            x2 = x1;
            x1 = adaptive ? round(xL + d) : (xL + d);
            f2 = f1;
            f1 = orc_criterion(pb, x1, adaptive, kernel, criterion, NULL);
            if (f1 < DBL_MAX) map_put(&m, x1, f1);
        }
        else
        {
            xU = x1;
            x1 = x2;
            x2 = adaptive ? floor(xU - d) : (xU - d);
            f1 = f2;
            f2 = orc_criterion(pb, x2, adaptive, kernel, criterion, NULL);
            if (f2 < DBL_MAX) map_put(&m, x2, f2);
        }
        iter = iter + 1;
        xopt = (f1 < f2) ? x1 : x2;
        d1 = f2 - f1;
    }
    (void)bw0;
    *bw_out = xopt;
    /* bandwidthCriterion(): sorted by bandwidth (BandwidthSelector.cpp:83-95) */
    for (int i = 1; i < m.n; i++)
        for (int j = i; j > 0 && m.bw[j - 1] > m.bw[j]; j--)
        {
            double tb = m.bw[j], tf = m.f[j];
            m.bw[j] = m.bw[j - 1]; m.f[j] = m.f[j - 1];
            m.bw[j - 1] = tb; m.f[j - 1] = tf;
        }
    return m.n;
}

/* -------------------------------------------------------------- diagnostic */

/* GWRBasic::CalcDiagnostic (GWRBasic.cpp:21-34). */
void orc_diagnostic(const orc_problem* pb, const double* betas, const double* shat, double* out)
{
    const int n_ = pb->n;
    double rss = rss_of(pb, pb->x, pb->p, betas);
    double n = (double)n_;
    double AIC = n * log(rss / n) + n * log(2 * M_PI) + n + shat[0];
    double AICc = n * log(rss / n) + n * log(2 * M_PI) + n * ((n + shat[0]) / (n - 2 - shat[0]));
    double edf = n - 2 * shat[0] + shat[1];
    double enp = 2 * shat[0] - shat[1];
    double mean = 0.0;
    for (int i = 0; i < n_; i++) mean += pb->y[i];
    mean /= n;
    double yss = 0.0;
    for (int i = 0; i < n_; i++) yss += (pb->y[i] - mean) * (pb->y[i] - mean);
    double r2 = 1 - rss / yss;
    double r2_adj = 1 - (1 - r2) * (n - 1) / (edf - 1);
    out[0] = rss; out[1] = AIC; out[2] = AICc; out[3] = enp; out[4] = edf; out[5] = r2; out[6] = r2_adj;
}

/* ------------------------------------------------------------------ MGWR */

/* GWRMultiscale (GWRMultiscale.cpp:68-317, serial forms :362-639): per-variable
   bandwidths by backfitting.  The per-variable criteria are GWRBasic's
   criteria of the one-column problem (x_i, y_i) (:560-638), the initial
   all-variable criterion is GWRBasic's on the centred X (:484-558), and the
   bandwidth searches are BandwidthSelector::optimize with MGWR's bounds. */

/* fitAllSerial with the hat matrix (:362-394): betas, betasSE = rowsum(ci^2),
   S0 rows si = x_i ci and SArray_k(i, :) = x(i, k) ci(k, :) (:216-224). */
static int mgwr_fit_all(const orc_problem* pb, double bw, int adaptive, int kernel, int hat, double* betas,
                        double* betas_se, double* S0, double* SA)
{
    const int n = pb->n, p = pb->p, T = orc_threads(pb);
    orc_ws* ws = (orc_ws*)malloc(sizeof(orc_ws) * (size_t)T);
    for (int t = 0; t < T; t++) ws_alloc(&ws[t], n, p, 1);
    int ok = 1;
#pragma omp parallel for num_threads(T) schedule(dynamic, 1) reduction(&& : ok)
    for (int i = 0; i < n; i++)
    {
        orc_ws* w = &ws[orc_thread_id()];
        orc_distance_row(pb, i, w->d);
        if (orc_weight(w->d, n, bw, adaptive, kernel, w->w) != 0 || local_solve(pb, pb->x, p, w) != 0)
        {
            ok = 0;
            continue;
        }
        for (int k = 0; k < p; k++) betas[(size_t)i + (size_t)k * n] = w->beta[k];
        if (!hat) continue;
        hat_row(pb, pb->x, p, i, w);
        for (int k = 0; k < p; k++)
        {
            double s = 0.0;
            for (int j = 0; j < n; j++) s += w->ci[k + (size_t)j * p] * w->ci[k + (size_t)j * p];
            betas_se[(size_t)i + (size_t)k * n] = s;
        }
        for (int j = 0; j < n; j++)
        {
            S0[(size_t)i + (size_t)j * n] = w->si[j];
            for (int k = 0; k < p; k++)
                SA[(size_t)k * n * n + (size_t)i + (size_t)j * n] =
                    pb->x[(size_t)i + (size_t)k * n] * w->ci[k + (size_t)j * p];
        }
    }
    for (int t = 0; t < T; t++) ws_free(&ws[t]);
    free(ws);
    return ok ? 0 : -1;
}

/* fitVarSerial (:420-482) on the one-column problem: betas and S rows si. */
static int mgwr_fit_var(const orc_problem* pb1, double bw, int adaptive, int kernel, int hat, double* beta,
                        double* S)
{
    const int n = pb1->n, T = orc_threads(pb1);
    orc_ws* ws = (orc_ws*)malloc(sizeof(orc_ws) * (size_t)T);
    for (int t = 0; t < T; t++) ws_alloc(&ws[t], n, 1, 1);
    int ok = 1;
#pragma omp parallel for num_threads(T) schedule(dynamic, 1) reduction(&& : ok)
    for (int i = 0; i < n; i++)
    {
        orc_ws* w = &ws[orc_thread_id()];
        orc_distance_row(pb1, i, w->d);
        if (orc_weight(w->d, n, bw, adaptive, kernel, w->w) != 0 || local_solve(pb1, pb1->x, 1, w) != 0)
        {
            ok = 0;
            continue;
        }
        beta[i] = w->beta[0];
        if (!hat) continue;
        hat_row(pb1, pb1->x, 1, i, w);
        for (int j = 0; j < n; j++) S[(size_t)i + (size_t)j * n] = w->si[j];
    }
    for (int t = 0; t < T; t++) ws_free(&ws[t]);
    free(ws);
    return ok ? 0 : -1;
}

/* C = A * B + A, all n x n column-major (the S * SArrayi + S update, :298-300). */
static void mat_mul_add(int n, const double* A, const double* B, double* C)
{
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++)
        {
            double s = 0.0;
            for (int k = 0; k < n; k++) s += A[(size_t)i + (size_t)k * n] * B[(size_t)k + (size_t)j * n];
            C[(size_t)i + (size_t)j * n] = s + A[(size_t)i + (size_t)j * n];
        }
}

static double mgwr_rss(int n, int p, const double* x, const double* y, const double* betas)
{
    double s = 0.0;
    for (int i = 0; i < n; i++)
    {
        double f = 0.0;
        for (int k = 0; k < p; k++) f += betas[(size_t)i + (size_t)k * n] * x[(size_t)i + (size_t)k * n];
        const double r = y[i] - f;
        s += r * r;
    }
    return s;
}

int orc_mgwr_fit(const orc_problem* pb0, const orc_mgwr_opts* o, orc_mgwr_out* out)
{
    const int n = pb0->n, p = pb0->p;
    const double maxd = orc_max_distance(pb0);
    /* centring of the predictors (:90-99) */
    double* xc = (double*)malloc(sizeof(double) * (size_t)n * (size_t)p);
    memcpy(xc, pb0->x, sizeof(double) * (size_t)n * (size_t)p);
    for (int k = o->has_intercept ? 1 : 0; k < p; k++)
        if (o->centered[k])
        {
            double m = 0.0;
            for (int i = 0; i < n; i++) m += xc[(size_t)i + (size_t)k * n];
            m /= n;
            for (int i = 0; i < n; i++) xc[(size_t)i + (size_t)k * n] -= m;
        }
    orc_problem pb = *pb0;
    pb.x = xc;
    double* bws = out->bws;
    int* init = (int*)malloc(sizeof(int) * (size_t)p);
    for (int k = 0; k < p; k++)
    {
        bws[k] = o->bw0[k];
        init[k] = o->init_type[k];
    }
    double* yi = (double*)malloc(sizeof(double) * (size_t)n);
    orc_problem pb1 = pb;
    pb1.p = 1;
    pb1.y = yi;
    int rc = 0;
    /* initial per-variable bandwidths (:104-133), against y itself */
    memcpy(yi, pb0->y, sizeof(double) * (size_t)n);
    for (int k = 0; k < p; k++)
    {
        if (init[k] != ORC_MGWR_INIT_NULL) continue;
        pb1.x = xc + (size_t)k * n;
        const int ad = o->adaptive[k];
        const double lo = o->has_lower ? o->lower : (ad ? o->adaptive_lower : maxd / 5000.0);
        const double hi = o->has_upper ? o->upper : (ad ? n : maxd);
        double b;
        /* BandwidthSelector::optimize throws "Invalid initial values." (BandwidthSelector.cpp:26-29) */
        if (orc_golden(&pb1, bws[k], ad, o->kernel[k], o->approach[k] == ORC_MGWR_CV ? ORC_CV : ORC_AIC, lo, hi, &b,
                       NULL, NULL, 0) < 0)
        {
            rc = -2;
            goto done;
        }
        bws[k] = b;
    }
    /* initial all-variable bandwidth (:135-155) with the first variable's weight */
    {
        const int ad = o->adaptive[0];
        const double lo = o->has_lower ? o->lower : (ad ? o->adaptive_lower : maxd / 5000.0);
        const double hi = o->has_upper ? o->upper : (ad ? n : maxd);
        if (orc_golden(&pb, bws[0], ad, o->kernel[0], o->approach[0] == ORC_MGWR_CV ? ORC_CV : ORC_AIC, lo, hi,
                       &out->init_bw, NULL, NULL, 0) < 0)
        {
            rc = -2; /* "Cannot select initial bandwidth." */
            goto done;
        }
    }
    {
        const int hat = o->has_hat_matrix;
        double* S0 = hat ? (double*)calloc((size_t)n * n, sizeof(double)) : NULL;
        double* SA = hat ? (double*)calloc((size_t)p * n * n, sizeof(double)) : NULL;
        double* S = hat ? (double*)calloc((size_t)n * n, sizeof(double)) : NULL;
        double* SAi = hat ? (double*)malloc(sizeof(double) * (size_t)n * n) : NULL;
        double* betas = out->betas;
        double* resid = (double*)malloc(sizeof(double) * (size_t)n);
        int* same = (int*)calloc((size_t)p, sizeof(int));
        /* backfitting (:208-317) */
        if (mgwr_fit_all(&pb, out->init_bw, o->adaptive[0], o->kernel[0], hat, betas, out->betas_se, S0, SA) != 0)
        {
            rc = -3;
            goto done2;
        }
        for (int i = 0; i < n; i++)
        {
            double f = 0.0;
            for (int k = 0; k < p; k++) f += betas[(size_t)i + (size_t)k * n] * xc[(size_t)i + (size_t)k * n];
            resid[i] = pb0->y[i] - f;
        }
        double RSS0 = 0.0, RSS1 = DBL_MAX, crit = DBL_MAX;
        for (int i = 0; i < n; i++) RSS0 += resid[i] * resid[i];
        int iter;
        for (iter = 1; iter <= o->max_iteration && crit > o->criterion_threshold; iter++)
        {
            for (int k = 0; k < p; k++)
            {
                const double* xk = xc + (size_t)k * n;
                for (int i = 0; i < n; i++) yi[i] = resid[i] + betas[(size_t)i + (size_t)k * n] * xk[i];
                pb1.x = xk;
                if (init[k] != ORC_MGWR_INIT_SPECIFIED)
                {
                    const int ad = o->adaptive[k];
                    /* mMaxDistances[k] is only filled for Null-initialised variables (:117); it
                       stays 0 for the others */
                    const double mdk = o->init_type[k] == ORC_MGWR_INIT_NULL ? maxd : 0.0;
                    const double lo = o->has_lower ? o->lower : (ad ? o->adaptive_lower : mdk / 5000.0);
                    const double hi = o->has_upper ? o->upper : (ad ? n : mdk);
                    double b = bws[k];
                    if (orc_golden(&pb1, bws[k], ad, o->kernel[k], o->approach[k] == ORC_MGWR_CV ? ORC_CV : ORC_AIC,
                                   lo, hi, &b, NULL, NULL, 0) < 0)
                    {
                        rc = -2;
                        goto done2;
                    }
                    if (fabs(b - bws[k]) > o->select_threshold[k])
                        same[k] = 0;
                    else if (++same[k] >= o->retry_times)
                        init[k] = ORC_MGWR_INIT_SPECIFIED;
                    bws[k] = b;
                }
                double* bk = betas + (size_t)k * n;
                if (mgwr_fit_var(&pb1, bws[k], o->adaptive[k], o->kernel[k], hat, bk, S) != 0)
                {
                    rc = -3;
                    goto done2;
                }
                if (hat)
                {
                    double* SAk = SA + (size_t)k * n * n;
                    for (size_t e = 0; e < (size_t)n * n; e++) SAi[e] = SAk[e] - S0[e];
                    mat_mul_add(n, S, SAi, SAk);
                    for (size_t e = 0; e < (size_t)n * n; e++) S0[e] = SAk[e] - SAi[e];
                }
                for (int i = 0; i < n; i++)
                {
                    double f = 0.0;
                    for (int q = 0; q < p; q++) f += betas[(size_t)i + (size_t)q * n] * xc[(size_t)i + (size_t)q * n];
                    resid[i] = pb0->y[i] - f;
                }
            }
            RSS1 = mgwr_rss(n, p, xc, pb0->y, betas);
            crit = o->criterion_type == ORC_MGWR_CVR ? fabs(RSS1 - RSS0) : sqrt(fabs(RSS1 - RSS0) / RSS1);
            RSS0 = RSS1;
        }
        out->iterations = iter - 1;
        out->rss = RSS0;
        /* diagnostics (:174-180, CalcDiagnostic :41-66) */
        double trS = 0.0, trStS = 0.0;
        if (hat)
        {
            for (int i = 0; i < n; i++) trS += S0[(size_t)i + (size_t)i * n];
            for (size_t e = 0; e < (size_t)n * n; e++) trStS += S0[e] * S0[e];
        }
        out->shat[0] = trS;
        out->shat[1] = trStS;
        double ym = 0.0, tss = 0.0;
        for (int i = 0; i < n; i++) ym += pb0->y[i];
        ym /= n;
        for (int i = 0; i < n; i++) tss += (pb0->y[i] - ym) * (pb0->y[i] - ym);
        const double nn = (double)n;
        const double edf = nn - 2 * trS + trStS;
        out->diag[0] = RSS0;
        out->diag[1] = nn * log(RSS0 / nn) + nn * log(2 * M_PI) + nn * ((nn + trS) / (nn - 2 - trS));
        out->diag[2] = 2 * trS - trStS;
        out->diag[3] = edf;
        out->diag[4] = 1 - RSS0 / tss;
        out->diag[5] = 1 - (1 - out->diag[4]) * (nn - 1) / (edf - 1);
    done2:
        free(S0);
        free(SA);
        free(S);
        free(SAi);
        free(resid);
        free(same);
    }
done:
    free(xc);
    free(init);
    free(yi);
    return rc;
}
