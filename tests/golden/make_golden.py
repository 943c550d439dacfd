"""Generate tests/golden/londonhp100.json from the reference's own test fixture.

Reads the reference checkout (argument 1, or the GWMODEL_REFERENCE environment
variable) -- the londonhp100 coordinates and data that test/testGWRBasic.cpp loads through
test/data/londonhp100.cpp:6-26 -- and records the known answers that
test/testGWRBasic.cpp asserts (absolute tolerance 1e-8), with the line each
comes from.  The GPU machine has no reference checkout, so the tests read this
JSON instead.

    python tests/golden/make_golden.py /path/to/libgwmodel
"""
import csv
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def read_csv(path, fields):
    with open(path, newline="") as f:
        rows = list(csv.DictReader(f))
    return [[float(r[k]) for k in fields] for r in rows]


def main(ref=None):
    ref = ref or os.environ.get("GWMODEL_REFERENCE")
    if not ref:
        sys.exit("usage: make_golden.py /path/to/libgwmodel (or set GWMODEL_REFERENCE)")
    data_dir = os.path.join(ref, "test", "data")
    coords = read_csv(os.path.join(data_dir, "londonhp100coords.csv"), ["x", "y"])
    data = read_csv(os.path.join(data_dir, "londonhp100data.csv"),
                    ["PURCHASE", "FLOORSZ", "UNEMPLOY", "PROF"])
    expected = {
        "adaptive_gaussian_bw36": {
            "source": "test/testGWRBasic.cpp:40-68",
            "bandwidth": 36, "adaptive": True, "kernel": "gaussian",
            "AIC": 2436.60445730413, "AICc": 2448.27206524754,
            "RSquare": 0.708010632044736, "RSquareAdjust": 0.674975341723766,
        },
        "fixed_gaussian_bw5000": {
            "source": "test/testGWRBasic.cpp:70-103",
            "bandwidth": 5000, "adaptive": False, "kernel": "gaussian",
            "AIC": 2437.649574267587, "AICc": 2447.676281164379,
            "RSquare": 0.701466295457, "RSquareAdjust": 0.673691594464,
        },
        "adaptive_gaussian_cv_search": {
            "source": "test/testGWRBasic.cpp:105-137",
            "adaptive": True, "kernel": "gaussian", "criterion": "CV",
            "selected_bandwidth": 67,
        },
        "variable_selection_aic": {
            "source": "test/testGWRBasic.cpp:139-184",
            "bandwidth": 36, "adaptive": True, "kernel": "gaussian", "threshold": 3.0,
            "criterion_list": [[[2], 2551.61359020599], [[3], 2551.30032201349],
                               [[1], 2468.93236280013], [[1, 3], 2452.86447942033],
                               [[1, 2], 2450.59642666509], [[1, 2, 3], 2452.80388934625]],
            "selected": [1, 3],
        },
        "cv_search_with_variable_selection": {
            "source": "test/testGWRBasic.cpp:186-240",
            "adaptive": True, "kernel": "gaussian", "criterion": "CV", "threshold": 3.0,
            "selected": [1, 3], "selected_bandwidth": 31.0,
            "AIC": 2435.8161441795, "AICc": 2445.49629974057,
            "RSquare": 0.706143867720706, "RSquareAdjust": 0.678982114793865,
        },
    }
    # test/testGWRMultiscale.cpp:31-32: y = PURCHASE, x = [1, FLOORSZ, PROF]; every section
    # uses a bisquare kernel, centres the two non-intercept columns and a select threshold of
    # 1e-5 per variable.  Bandwidths are asserted to 0.1 (fixed) or exactly (adaptive), the
    # diagnostics to 1e-6.  "criterion" is the back-fitting convergence measure; sections that
    # do not set it use the default, dCVR.
    mgwr_common = {"x_columns": [1, 3], "y_column": 0, "kernel": "bisquare",
                   "centered": [False, True, True], "select_threshold": 1e-5}
    mgwr = {
        "fixed_null_cv_hat": {
            "source": "test/testGWRMultiscale.cpp:45-88",
            "adaptive": False, "bw0": 0, "init": "Null", "approach": "CV",
            "hat_matrix": True, "criterion": "dCVR", "retry_times": 0,
            "bandwidths": [4623.78, 12665.70, 12665.70], "bandwidth_tol": 0.1,
            "AICc": 2437.09277417389, "RSquare": 0.744649364494,
            "RSquareAdjust": 0.712344894394,
        },
        "adaptive_initial_aic_hat_dcvr": {
            "source": "test/testGWRMultiscale.cpp:90-133",
            "adaptive": True, "bw0": 36, "init": "Initial", "approach": "AIC",
            "hat_matrix": True, "criterion": "dCVR", "retry_times": 5,
            "bandwidths": [45, 98, 98], "bandwidth_tol": 0.1,
            "AICc": 2437.935218705351, "RSquare": 0.7486787930045755,
            "RSquareAdjust": 0.7118919517893492,
        },
        "adaptive_null_cv_nohat": {
            "source": "test/testGWRMultiscale.cpp:135-173",
            "adaptive": True, "bw0": 0, "init": "Null", "approach": "CV",
            "hat_matrix": False, "criterion": "dCVR", "retry_times": 0,
            "bandwidths": [35, 98, 98], "bandwidth_tol": 0.0,
            "RSquare": 0.757377391669,
        },
        "adaptive_initial_cv_hat_cvr": {
            "source": "test/testGWRMultiscale.cpp:175-218",
            "adaptive": True, "bw0": 36, "init": "Initial", "approach": "CV",
            "hat_matrix": True, "criterion": "CVR", "retry_times": 5,
            "bandwidths": [35, 98, 98], "bandwidth_tol": 0.0,
            "AICc": 2438.256543496552, "RSquare": 0.757377391669,
            "RSquareAdjust": 0.715598248225,
        },
        "adaptive_null_cv_hat_cvr_bounds": {
            "source": "test/testGWRMultiscale.cpp:220-258",
            "adaptive": True, "bw0": 36, "init": "Null", "approach": "CV",
            "hat_matrix": True, "criterion": "CVR", "retry_times": 5,
            "lower": 50, "upper": 100,
            "bandwidths": [52, 99, 99], "bandwidth_tol": 0.0,
        },
    }
    for case in mgwr.values():
        for k, v in mgwr_common.items():
            case.setdefault(k, v)
    out = {
        "about": "londonhp100 fixture of libgwmodel test/data (x, y; PURCHASE, FLOORSZ, "
                 "UNEMPLOY, PROF) and the known answers of test/testGWRBasic.cpp and "
                 "test/testGWRMultiscale.cpp; generated by tests/golden/make_golden.py",
        "tolerance_abs": 1e-8,
        "coords": coords,
        "data": data,
        "expected": expected,
        "mgwr_tolerance_abs": 1e-6,
        "mgwr": mgwr,
    }
    with open(os.path.join(HERE, "londonhp100.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", os.path.join(HERE, "londonhp100.json"), len(coords), "rows")


if __name__ == "__main__":
    main(*sys.argv[1:])
