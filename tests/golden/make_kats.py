"""Writes tests/golden/kats.json: the known-answer cases of the reference's own
unit tests for the metric spaces, transcribed with their file:line.

The expected values are the reference tests' own expressions (e.g.
``2*M_PI - 4.0``) evaluated in IEEE double, the arithmetic the C++ tests use;
they are stored as hex floats so the comparison stays bit-exact.  Run from the
repository root:  python tests/golden/make_kats.py [output path]
"""
import json
import math
import os
import sys

PI = math.pi


def h(x: float) -> str:
    return float(x).hex()


def axis_angle_quat(angle, axis):
    """Eigen::AngleAxisd -> Quaterniond coefficients (x, y, z, w)."""
    n = math.sqrt(sum(a * a for a in axis))
    ax = [a / n for a in axis]
    s = math.sin(angle / 2)
    return [ax[0] * s, ax[1] * s, ax[2] * s, math.cos(angle / 2)]


cases = []
# test/lp_space_test.cpp:39-50  LPSpace<double,3,2> distance, exact ==
cases.append({"src": "test/lp_space_test.cpp:39-50", "op": "distance", "metric": 0, "dim": 3,
              "a": [1, 2, 3], "b": [1, 0, -1], "expect": h(math.sqrt(0.0 + 2.0 * 2.0 + 4.0 * 4.0)), "tol": 0})
# test/lp_space_test.cpp:53-66  interpolate(a, b, 0.1) == (1, 1.8, 2.6), exact ==
cases.append({"src": "test/lp_space_test.cpp:53-66", "op": "interpolate", "metric": 0, "dim": 3,
              "a": [1, 2, 3], "b": [1, 0, -1], "t": 0.1, "expect": [h(1.0), h(1.8), h(2.6)], "tol": 0})
# test/so2_space_test.cpp:39-50  SO2Space<double> scalar distances, exact ==
for a, b, e in [(1.0, 1.0, 0.0), (0.0, 2.0, 2.0), (2.0, 0.0, 2.0), (-1.0, 3.0, 2 * PI - 4.0), (3.0, -1.0, 2 * PI - 4.0)]:
    cases.append({"src": "test/so2_space_test.cpp:39-50", "op": "distance", "metric": 1, "dim": 1,
                  "a": [a], "b": [b], "expect": h(e), "tol": 0})
# test/so2_space_test.cpp:53-65  SO2LPSpace<double,3,1>, exact ==
cases.append({"src": "test/so2_space_test.cpp:53-65", "op": "distance", "metric": 1, "dim": 3,
              "a": [1, 2, 3], "b": [1, 0, -1], "expect": h(0.0 + 2.0 + 2 * PI - 4), "tol": 0})
# test/so2_space_test.cpp:68-83  SO2 interpolate incl. extrapolation, exact ==
for a, b, t, e in [(1.0, 1.0, 0.0, 1.0), (1.0, 1.0, 3.0, 1.0), (1.0, 2.0, 0.5, 1.5), (1.0, 2.0, -3.0, -2.0),
                   (-1.0, 2.0, 4.0, 11.0 - 4 * PI), (5 * PI / 6, -5 * PI / 6, 1.0, -5 * PI / 6),
                   (5 * PI / 6, -5 * PI / 6, 2.0, -3 * PI / 6), (-5 * PI / 6, 5 * PI / 6, 2.0, 3 * PI / 6)]:
    cases.append({"src": "test/so2_space_test.cpp:68-83", "op": "interpolate", "metric": 1, "dim": 1,
                  "a": [h(a)], "b": [h(b)], "t": h(t), "expect": [h(e)], "tol": 0})
# test/so3_space_test.cpp:39-56  acos(|a.b|) = 3/2 for angles -1 and 2 about (-1,2,3), tol 1e-10
axis = [-1, 2, 3]
cases.append({"src": "test/so3_space_test.cpp:39-56", "op": "distance", "metric": 2, "dim": 4,
              "a": [h(v) for v in axis_angle_quat(-1.0, axis)], "b": [h(v) for v in axis_angle_quat(2.0, axis)],
              "expect": h(1.5), "tol": 1e-10})
# test/so3_space_test.cpp:58-78  slerp at t=0.1 between angles 0.5 and 2.5: angle 0.7, same axis
cases.append({"src": "test/so3_space_test.cpp:58-78", "op": "slerp_angle", "metric": 2, "dim": 4,
              "a": [h(v) for v in axis_angle_quat(0.5, axis)], "b": [h(v) for v in axis_angle_quat(2.5, axis)],
              "t": 0.1, "expect_angle": 0.5 + 2 * 0.1, "axis": axis, "tol": 1e-10, "axis_tol": 1e-15})
# test/se3_space_test.cpp:45-89  weights (1,1),(5,2),(11,1),(1,13), tol 1e-9
for w0, w1 in [(1, 1), (5, 2), (11, 1), (1, 13)]:
    qa = axis_angle_quat(-1.0, axis)
    qb = axis_angle_quat(2.0, axis)
    cases.append({"src": "test/se3_space_test.cpp:45-89", "op": "distance", "metric": 3, "dim": 7, "w": [w0, w1],
                  "a": [h(v) for v in qa + [1, 2, 3]], "b": [h(v) for v in qb + [1, 0, -1]],
                  "expect": h(3.0 / 2 * w0 + math.sqrt(0.0 + 2.0 * 2.0 + 4.0 * 4.0) * w1), "tol": 1e-9})
# test/se3_space_test.cpp:92-117  interpolate: translation exact (1, 1.8, 2.6), rotation angle 0.7
qa = axis_angle_quat(0.5, axis)
qb = axis_angle_quat(2.5, axis)
cases.append({"src": "test/se3_space_test.cpp:92-117", "op": "se3_interpolate", "metric": 3, "dim": 7, "w": [1, 1],
              "a": [h(v) for v in qa + [1, 2, 3]], "b": [h(v) for v in qb + [1, 0, -1]], "t": 0.1,
              "expect_t": [h(1.0), h(1.8), h(2.6)], "expect_angle": 0.7, "axis": axis, "tol": 1e-10,
              "axis_tol": 1e-15})
# test/scaled_space_test.cpp:40-52  ScaledSpace<LPSpace<double,3,2>, ratio<5,2>>, exact ==
cases.append({"src": "test/scaled_space_test.cpp:40-52", "op": "scaled_distance", "metric": 0, "dim": 3,
              "a": [1, 2, 3], "b": [1, 0, -1], "scale": 2.5,
              "expect": h(math.sqrt(0.0 + 2.0 * 2.0 + 4.0 * 4.0) * 5 / 2), "tol": 0})

# an output path may be given (the reproducibility test writes to a temporary file)
out = sys.argv[1] if len(sys.argv) > 1 else os.path.join(os.path.dirname(os.path.abspath(__file__)), "kats.json")
with open(out, "w") as f:
    json.dump({"generated_by": "tests/golden/make_kats.py", "cases": cases}, f, indent=1)
print("wrote", out, len(cases), "cases")
