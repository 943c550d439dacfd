// golden.h -- golden-section bandwidth search, BandwidthSelector::optimize
// (BandwidthSelector.cpp:6-81), shared by the gwm::GWRBasic facade and the
// engine's device-resident search.
#pragma once

#include <cfloat>
#include <cmath>
#include <map>
#include <stdexcept>

namespace gwgpu {

// crit(bw) evaluates one bandwidth (DBL_MAX when invalid); ok() reports the
// algorithm status after each evaluation (false once cancelled).  Returns
// false when the search stopped on a bad status: the caller keeps its initial
// bandwidth, as optimize() returns mBandwidth.  record receives every finite
// criterion by bandwidth (insert-or-assign, sorted by the map).
template <class Crit, class Ok>
bool golden_section(double lower, double upper, bool adaptive, Crit&& crit, Ok&& ok, double& xopt,
                    std::map<double, double>& record)
{
    double xU = upper, xL = lower;
    const double eps = 1e-4;
    const double R = (std::sqrt(5) - 1) / 2;
    int iter = 0;
    double d = R * (xU - xL);
    double x1 = adaptive ? std::floor(xL + d) : (xL + d);
    double x2 = adaptive ? std::round(xU - d) : (xU - d);
    double f1 = crit(x1);
    bool s1 = ok();
    double f2 = crit(x2);
    bool s2 = ok();
    if (!(s1 && s2)) return false;
    if (f1 == DBL_MAX && f2 == DBL_MAX) throw std::runtime_error("Invalid initial values.");
    if (f1 < DBL_MAX) record[x1] = f1;
    if (f2 < DBL_MAX) record[x2] = f2;
    double d1 = f2 - f1;
    xopt = f1 < f2 ? x1 : x2;
    const double ea = 100;
    while (s1 && s2 && std::fabs(d) > eps && std::fabs(d1) > eps && iter < ea) {
        d = R * d;
        if (f1 < f2) {
            xL = x2;
            x2 = x1;
            x1 = adaptive ? std::round(xL + d) : (xL + d);
            f2 = f1;
            f1 = crit(x1);
            s1 = ok();
            if (f1 < DBL_MAX) record[x1] = f1;
        } else {
            xU = x1;
            x1 = x2;
            x2 = adaptive ? std::floor(xU - d) : (xU - d);
            f1 = f2;
            f2 = crit(x2);
            s2 = ok();
            if (f2 < DBL_MAX) record[x2] = f2;
        }
        iter = iter + 1;
        xopt = (f1 < f2) ? x1 : x2;
        d1 = f2 - f1;
    }
    return s1 && s2;
}

}  // namespace gwgpu
