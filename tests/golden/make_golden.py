"""Generate tests/golden/londonhp100.json from the reference's own test fixture.

Reads the reference checkout (argument 1, default /root/reference) -- the
londonhp100 coordinates and data that test/testGWRBasic.cpp loads through
test/data/londonhp100.cpp:6-26 -- and records the known answers that
test/testGWRBasic.cpp asserts (absolute tolerance 1e-8), with the line each
comes from.  The GPU machine has no reference checkout, so the tests read this
JSON instead.

    python tests/golden/make_golden.py [/path/to/reference]
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


def main(ref="/root/reference"):
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
    out = {
        "about": "londonhp100 fixture of libgwmodel test/data (x, y; PURCHASE, FLOORSZ, "
                 "UNEMPLOY, PROF) and the known answers of test/testGWRBasic.cpp; "
                 "generated by tests/golden/make_golden.py",
        "tolerance_abs": 1e-8,
        "coords": coords,
        "data": data,
        "expected": expected,
    }
    with open(os.path.join(HERE, "londonhp100.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", os.path.join(HERE, "londonhp100.json"), len(coords), "rows")


if __name__ == "__main__":
    main(*sys.argv[1:])
