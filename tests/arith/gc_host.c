/*
 * gc_host.c -- test helper: the engine's great-circle arithmetic
 * (libgwmodel_gb300/csrc/gw_arith.h) compiled for the host, so tests can
 * check the correctly rounded sin/cos/atan against an arbitrary-precision
 * reference and against the platform libm, and can recompute the exact
 * distances the GPU select ranks.  Built by the tests with
 * gcc -O2 -ffp-contract=off.
 */
#include <math.h>

#include "../../libgwmodel_gb300/csrc/gw_arith.h"

void gc_sincos_cr(const double* x, double* s, double* c, int n)
{
    for (int i = 0; i < n; i++) gw_sincos_cr(x[i], s + i, c + i);
}

void gc_atan_cr(const double* x, double* a, int n)
{
    for (int i = 0; i < n; i++) a[i] = gw_atan_cr(x[i]);
}

/* SpGcdist(data lon, focus lon, data lat, focus lat) for every data point j,
 * radians rounded as the engine stores them (lon * (M_PI / 180)). */
void gc_row_cr(const double* lon, const double* lat, int n, int focus, double* out)
{
    const double DE2RA = M_PI / 180;
    const double fu = lon[focus], fv = lat[focus];
    for (int j = 0; j < n; j++)
        out[j] = gw_gc_dist(lon[j], fu, lat[j], fv, lon[j] * DE2RA, fu * DE2RA, lat[j] * DE2RA, fv * DE2RA);
}
