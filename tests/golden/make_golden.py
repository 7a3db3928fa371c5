"""Writes the golden fixtures under tests/golden/ from the reference's own tests and data.

Run once where the rti sources are checked out, with their root as the one
required argument (``python tests/golden/make_golden.py <rti-root>``); the
fixtures it writes are committed and travel with the repository.

* area_inside_cases.json -- the 37 known-answer cases of
  test/rti/geo/disc_bounding_box_intersector.cpp, with the expected value
  evaluated exactly as each test expression does (float or double arithmetic)
  and each test's own tolerance (0 = ASSERT_EQ).
* local_intersector_cases.json -- the 9 hand-built hit/miss cases of
  test/rti/trace/local_intersector.cpp:14-129.
* radiosity_ar45_sp{1,0.1,0.01}.txt -- verification/radiosity/analytical_solution/
  sp.{1,0.1,0.01}.data: analytical radiosity wall flux (normalised depth,
  max-normalised flux) for a cylinder of radius 0.5 and length 45.
"""
from __future__ import annotations

import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = ""  # the rti source root, from the command line (main)
TEST = "test/rti/geo/disc_bounding_box_intersector.cpp"

f32 = np.float32
PI_F = f32(math.pi)          # (float) rti::util::pi()


def exact(v):
    return {"expected": float(v), "tol": 0.0}


def approx(v, tol):
    return {"expected": float(v), "tol": tol}


def seg_x_right(r, x):       # test_1 lines 98-122: alpha = 2 acos((1.0 - x)/r)
    alpha = 2 * math.acos((1.0 - float(f32(x))) / float(r))
    return float(r) * float(r) * math.pi - float(f32(r) * f32(r) / f32(2)) * (alpha - math.sin(alpha))


def seg_x_left(r, x):        # test_1 lines 134-148: alpha = 2 acos((1.0 + x)/r)
    alpha = 2 * math.acos((1.0 + float(f32(x))) / float(r))
    return float(r) * float(r) * math.pi - float(f32(r) * f32(r) / f32(2)) * (alpha - math.sin(alpha))


def tilted_bottom():         # test_2 lines 226-242, evaluated in float as written
    r, d = f32(1), f32(0.7)
    alpha = f32(2) * np.arccos(np.sqrt(d * d * f32(2)) / r)
    alpha = f32(2 * math.pi - float(alpha))
    return r * r / f32(2) * (alpha - np.sin(alpha))


B1 = [-1, -1, 1, 1]
B2 = [-2, -4, 8, 1]
B3 = [-100, -100, 0, 0]
B4 = [-2, -4, 8, 1]

# (line, name, box [xmin ymin xmax ymax], disc [x y z r], normal, expectation)
CASES = [
    (34, "disc_fully_inside_r_1", B1, [0, 0, 0, 1], [0, 0, 1], exact(PI_F)),
    (42, "disc_fully_inside_r_0_5", B1, [0.2, 0.2, 0, 0.5], [0, 0, 1], exact(f32(0.5) * f32(0.5) * PI_F)),
    (50, "disc_fully_outside_x_direction", B1, [2, 0, 0, 1], [0, 0, 1], exact(0)),
    (58, "disc_fully_outside_y_direction", B1, [0, 2, 0, 1], [0, 0, 1], exact(0)),
    (66, "disc_inside_parallel_to_bounding_box_x_direction", B1, [0.5, 0, 0, 1], [1, 0, 0], exact(PI_F)),
    (74, "disc_outside_parallel_to_bounding_box_x_direction", B1, [1.5, 0, 0, 1], [1, 0, 0], exact(0)),
    (82, "disc_fully_inside_tilted_close_to_boundary", B1, [0.2, 0, 0, 1], [1, 0, 1], exact(PI_F)),
    (90, "disc_half_inside_x_direction_right", B1, [1, 0, 0, 1], [0, 0, 1], exact(f32(0.5) * PI_F)),
    (98, "disc_a_bit_outside_x_direction_right", B1, [0.5, 0, 0, 1], [0, 0, 1], approx(seg_x_right(1, 0.5), 1e-7)),
    (110, "disc_almost_entirely_outside_x_direction_right", B1, [1.9, 0, 0, 1], [0, 0, 1],
     approx(seg_x_right(1, 1.9), 1e-6)),
    (126, "disc_half_inside_x_direction_left", B1, [-1, 0, 0, 1], [0, 0, 1], exact(f32(0.5) * PI_F)),
    (134, "disc_almost_entirely_outside_x_direction_left", B1, [-1.9, 0, 0, 1], [0, 0, 1],
     approx(seg_x_left(1, -1.9), 1e-6)),
    (150, "disc_half_inside_y_direction_top", B1, [0, 1, 0, 1], [0, 0, 1], exact(f32(0.5) * PI_F)),
    (158, "disc_half_inside_y_direction_bottom", B1, [1, 0, 0, 1], [0, 0, 1], exact(f32(0.5) * PI_F)),
    (166, "disc_half_inside_tilted_y_direction_bottom", B1, [1, 0, 0, 1], [0, 1, 1], exact(f32(0.5) * PI_F)),
    (174, "disc_inside_parallel_to_bounding_box_y_direction", B1, [0, 0.8, 0, 1], [0, 1, 0], exact(PI_F)),
    (183, "t2_disc_half_inside_x_direction_right", B2, [8, -1, 0, 1], [0, 1, 1], exact(0.5 * float(PI_F))),
    (194, "t2_disc_fully_inside_x_direction_right", B2, [7.18, -1, 0, 1], [1, 1, 1], exact(PI_F)),
    (202, "t2_disc_half_inside_x_direction_left", B2, [-2, -1, 0, 1], [0, 0, 1], exact(0.5 * float(PI_F))),
    (210, "t2_disc_half_inside_y_direction_bottom", B2, [3, -4, 0, 1], [0, 0, 1], exact(0.5 * float(PI_F))),
    (218, "t2_disc_half_inside_y_direction_top", B2, [3, 1, 0, 1], [0, 0, 1], exact(0.5 * float(PI_F))),
    (226, "t2_disc_mostly_inside_tilted_y_direction_bottom", B2, [3, float(f32(-4) + f32(0.7)), 0, 1],
     [0.6, -1, 0.8], approx(tilted_bottom(), 1e-6)),
    (244, "t2_corner_top_right", B2, [8, 1, 0, 1], [0, 0, 1], approx(f32(0.25) * PI_F, 1e-6)),
    (254, "t2_corner_bottom_right", B2, [8, -4, 0, 1], [0, 0, 1], approx(f32(0.25) * PI_F, 1e-6)),
    (264, "t2_corner_bottom_left", B2, [-2, -4, 0, 1], [0, 0, 1], approx(f32(0.25) * PI_F, 1e-6)),
    (274, "t2_corner_top_left", B2, [-2, 1, 0, 1], [0, 0, 1], approx(f32(0.25) * PI_F, 1e-6)),
    (285, "t3_corner_most_simple", B3, [0, 0, 0, 1], [0, 0, 1], approx(PI_F / f32(4), 1e-6)),
    (296, "t3_corner_complex", B3, [-1, -4, 0, 8], [-1, -1, 1], approx(94.139436, 2e-3)),
    (311, "t4_top_right_corner_1", B4, [9.35, 1.5, 0, 2], [0, 0, 1], approx(0.349293, 1e-3)),
    (322, "t4_top_right_corner_2", B4, [9.35, 0.5, 0, 2], [0, 0, 1], approx(0.978276, 1e-3)),
    (333, "t4_top_right_corner_3", B4, [7.65, 1.5, 0, 2], [0, 0, 1], approx(2.673503, 1e-3)),
    (344, "t4_top_right_corner_4", B4, [7.65, 0.5, 0, 2], [0, 0, 1], approx(5.002261, 1e-3)),
    (355, "t4_bottom_right_corner", B4, [7.65, -4.33, 1, 2], [-0.79, 0.43, 0.11], approx(1.381609, 1e-3)),
    (365, "t4_bottom_left_corner", B4, [-1.82, -4.3, 2, 2], [-0.84, -0.53, -0.21], approx(0.806725, 1e-3)),
    (375, "t4_top_left_corner", B4, [-2.12, 1.43, 3, 2], [-0.65, 0.47, -0.84], approx(1.422461, 1e-3)),
    (386, "t4_large_disc", B4, [-12.11, -2.01, 1, 20], [0.23, 0.99, 0.45], approx(86.310325, 1e-2)),
    (397, "t4_huge_disc", B4, [-12.11, -2.01, 1, 30], [0.23, 0.99, 0.45], approx(123.516791, 2e-2)),
]

LI = "test/rti/trace/local_intersector.cpp"
# (line, name, org, dir, disc, normal, expected) -- dir and normal are normalised in float first
LOCAL = [
    (14, "simple_hit_front", [0, 0, 0], [0, 1, 0], [1, 10, 0, 2], [0, -1, 0], True),
    (27, "simple_hit_back", [0, 0, 0], [0, 1, 0], [1, 10, 0, 2], [0, 1, 0], False),
    (40, "simple_miss", [0, 0, 0], [0, 1, 1], [1, 10, 0, 2], [0, -1, 0], False),
    (53, "simple_parallel_miss", [0, 0, 0], [0, 1, 0], [1, 10, 0, 2], [-1, 0, 0], False),
    (66, "almost_parallel_miss", [0, 0, 0], [0, 1, 0], [1, 10, 0, 2], [-1, -0.01, 0], False),
    (79, "some_hit", [2, 10, 1.5], [0.133, -1, 0.05], [3, 5, 2, 2], [-1, 1.5, 0.5], True),
    (92, "miss_by_shooting_away", [2, 10, 1.5], [-0.2, 1, -0.21], [3, 5, 2, 2], [-1, 1.5, 0.5], False),
    (105, "tight_miss", [2, 10, 1.5], [-0.125, -1, 0.05], [3, 5, 2, 2], [-1, 1.5, 0.5], False),
    (118, "miss_by_starting_at_the_wrong_side_and_shooting_away", [1, 1, 1], [0, -1, 0], [3, 10, 2, 2],
     [0, 1, 0], False),
]


def normalize_f32(v):
    v = np.asarray(v, dtype=np.float32)
    n = np.sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])
    return [float(v[0] / n), float(v[1] / n), float(v[2] / n)]


def main():
    global REF
    if len(sys.argv) != 2:
        raise SystemExit("usage: make_golden.py <rti source root>")
    REF = sys.argv[1]
    src = os.path.join(REF, TEST)
    if not os.path.exists(src):
        raise SystemExit(f"reference tests not found under {REF}")
    text = open(src).read().splitlines()
    area = []
    for line, name, box, disc, normal, exp in CASES:
        assert "TEST_F" in text[line - 1], (line, text[line - 1])
        area.append({"source": f"{TEST}:{line}", "name": name, "box": box,
                     "disc": [float(f32(x)) for x in disc], "normal": [float(f32(x)) for x in normal], **exp})
    json.dump(area, open(os.path.join(HERE, "area_inside_cases.json"), "w"), indent=1)

    ltext = open(os.path.join(REF, LI)).read().splitlines()
    local = []
    for line, name, org, dr, disc, normal, expected in LOCAL:
        assert "TEST(" in ltext[line - 1], (line, ltext[line - 1])
        local.append({"source": f"{LI}:{line}", "name": name, "org": org, "dir": normalize_f32(dr),
                      "disc": [float(f32(x)) for x in disc], "normal": normalize_f32(normal),
                      "expected": expected})
    json.dump(local, open(os.path.join(HERE, "local_intersector_cases.json"), "w"), indent=1)

    for sp in ("1", "0.1", "0.01"):
        data = os.path.join(REF, "verification/radiosity/analytical_solution", f"sp.{sp}.data")
        rows = [ln.split() for ln in open(data) if ln.strip() and not ln.startswith("#")]
        with open(os.path.join(HERE, f"radiosity_ar45_sp{sp}.txt"), "w") as f:
            f.write(f"# verification/radiosity/analytical_solution/sp.{sp}.data (cylinder r=0.5, length 45)\n")
            f.write("# normalised_depth max_normalised_wall_flux\n")
            for a, b in rows:
                f.write(f"{a} {b}\n")
    print(f"wrote {len(area)} area cases, {len(local)} local-intersector cases, 3 radiosity curves")


if __name__ == "__main__":
    main()
