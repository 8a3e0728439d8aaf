"""Writes tests/golden/known_answers.json: the reference's GJK/EPA known answers, restated.

Each case cites the reference test it restates (file:line under the reference project). Shapes:
  ["aabb", min3, max3]
  ["obb", center3, rot, half3]           rot = null or [angle_rad, axis3] (axis normalised)
  ["mesh", spec, pos3, rot]              spec = ["box", hx, hy, hz] | ["sphere", r] | ["pyramid", b, h]
GJK cases give the expected boolean ("hit") and whether the reversed order is checked too.
EPA cases give an expected depth with its tolerance and optional direction/MTV/symmetry checks.
Run: python tests/golden/make_known_answers.py
"""
import json
import math
import os

PI = math.pi


def aabb(mn, mx):
    return ["aabb", list(map(float, mn)), list(map(float, mx))]


def obb(c, half, rot=None):
    return ["obb", list(map(float, c)), rot, list(map(float, half))]


def rot(angle, axis):
    n = math.sqrt(sum(a * a for a in axis))
    return [angle, [a / n for a in axis]]


def box(pos, h=(1.0, 1.0, 1.0), r=None):
    return ["mesh", ["box", *map(float, h)], list(map(float, pos)), r]


def sphere(pos, radius=1.0):
    return ["mesh", ["sphere", float(radius)], list(map(float, pos)), None]


def pyramid(pos, r=None):
    return ["mesh", ["pyramid", 1.0, 2.0], list(map(float, pos)), r]


U = ([-1, -1, -1], [1, 1, 1])
I3 = (1, 1, 1)
Z45 = rot(PI / 4, (0, 0, 1))
Z90 = rot(PI / 2, (0, 0, 1))
X90 = rot(PI / 2, (1, 0, 0))
Z180 = rot(PI, (0, 0, 1))
G = "tests/gjk/gjk_test.cpp"
E = "tests/epa/epa_test.cpp"


def gjk(line, a, b, hit, both=False):
    return {"src": f"{G}:{line}", "a": a, "b": b, "hit": hit, "both_orders": both}


GJK = [
    gjk(20, aabb(*U), aabb([0.5, -1, -1], [2.5, 1, 1]), True),
    gjk(28, aabb(*U), aabb([2, -1, -1], [4, 1, 1]), False),
    gjk(36, aabb(*U), aabb([-1, 2, -1], [1, 4, 1]), False),
    gjk(44, aabb(*U), aabb([-1, -1, 2], [1, 1, 4]), False),
    gjk(52, aabb([-3] * 3, [3] * 3), aabb(*U), True, both=True),
    gjk(61, aabb(*U), aabb([100, -1, -1], [102, 1, 1]), False),
    gjk(68, aabb(*U), aabb(*U), True),
    gjk(75, aabb([0] * 3, [2] * 3), aabb([1] * 3, [3] * 3), True),
    gjk(83, aabb(*U), aabb([5] * 3, [7] * 3), False),
    gjk(95, obb([0, 0, 0], I3), obb([1.5, 0, 0], I3), True),
    gjk(103, obb([0, 0, 0], I3), obb([3, 0, 0], I3), False),
    gjk(111, obb([0, 0, 0], I3), obb([0, 0, 0], I3, Z45), True),
    gjk(121, obb([0, 0, 0], I3), obb([1, 0, 0], I3, Z45), True),
    gjk(132, obb([0, 0, 0], I3), obb([3, 0, 0], I3, Z45), False),
    gjk(143, obb([0, 0, 0], (2, 0.2, 0.2)), obb([0, 0, 0], (2, 0.2, 0.2), Z90), True),
    gjk(153, obb([0, 0, 0], (2, 0.2, 0.2)), obb([0, 3, 0], (2, 0.2, 0.2), Z90), False),
    gjk(167, obb([0, 0, 0], I3), obb([0.5, 0.5, 0.5], I3, X90), True),
    gjk(177, obb([0, 0, 0], (3, 0.3, 3)), obb([0, 0, 0], (0.3, 3, 0.3)), True),
    gjk(185, obb([0, 0, 0], (3, 0.3, 3)), obb([5, 0, 0], (0.3, 3, 0.3)), False),
    gjk(193, obb([0, 0, 0], I3), obb([1.5, 1.5, 1.5], I3), True),
    gjk(201, obb([0, 0, 0], I3), obb([3, 3, 3], I3), False),
    gjk(213, obb([0, 0, 0], I3), aabb([0.5, -1, -1], [2.5, 1, 1]), True, both=True),
    gjk(221, obb([0, 0, 0], I3), aabb([2.5, -1, -1], [4.5, 1, 1]), False, both=True),
    gjk(229, obb([1, 0, 0], I3, Z45), aabb(*U), True, both=True),
    gjk(240, obb([5, 0, 0], I3, Z45), aabb(*U), False, both=True),
    gjk(251, obb([0, 0, 0], (0.5, 0.5, 0.5)), aabb([-2] * 3, [2] * 3), True, both=True),
    gjk(264, aabb(*U), aabb([0.5, -1, -1], [2.5, 1, 1]), True, both=True),
    gjk(271, aabb(*U), aabb([3, -1, -1], [5, 1, 1]), False, both=True),
    gjk(278, obb([0, 0, 0], I3), obb([1, 1, 0], I3, rot(PI / 6, (1, 1, 0))), True, both=True),
    gjk(287, obb([0, 0, 0], I3), obb([4, 0, 0], I3), False, both=True),
    gjk(294, aabb(*U), aabb([3, -1, -1], [5, 1, 1]), False),
    gjk(306, box([0, 0, 0]), box([1.5, 0, 0]), True),
    gjk(315, box([0, 0, 0]), box([3, 0, 0]), False),
    gjk(324, box([0, 0, 0], (3, 3, 3)), box([0, 0, 0], (0.5, 0.5, 0.5)), True, both=True),
    gjk(335, box([0, 0, 0]), box([0, 0, 0]), True),
    gjk(343, box([0, 0, 0]), box([1, 0, 0], r=Z45), True),
    gjk(354, box([0, 0, 0]), box([3, 0, 0], r=Z45), False),
    gjk(365, sphere([0, 0, 0]), sphere([1.5, 0, 0]), True),
    gjk(374, sphere([0, 0, 0]), sphere([3, 0, 0]), False),
    gjk(383, box([0, 0, 0]), sphere([1.5, 0, 0]), True, both=True),
    gjk(394, box([0, 0, 0]), sphere([3, 0, 0]), False, both=True),
    gjk(405, box([0, 0, 0]), box([1.5, 0, 0]), True, both=True),
    gjk(413, box([0, 0, 0]), box([4, 0, 0]), False, both=True),
    gjk(421, box([0, 0, 0]), box([4, 0, 0]), False),
    gjk(434, pyramid([0, 0, 0]), pyramid([0, 0, 0]), True),
    gjk(442, pyramid([0, 0, 0]), pyramid([0, 1.5, 0]), True),
    gjk(451, pyramid([0, 0, 0]), pyramid([0, 4, 0]), False),
    gjk(460, pyramid([0, 0, 0]), pyramid([4, 0, 0]), False),
    gjk(469, pyramid([0, 0, 0]), pyramid([0, 3, 0], r=Z180), True),
    gjk(481, pyramid([0, 0, 0]), pyramid([0, 6, 0], r=Z180), False),
    gjk(491, pyramid([0, 0, 0]), box([0, 0, 0]), True, both=True),
    gjk(502, pyramid([0, 0, 0]), box([0, -3, 0]), False, both=True),
    gjk(513, pyramid([0, 0, 0]), sphere([0, 1, 0]), True, both=True),
    gjk(524, pyramid([0, 0, 0]), sphere([0, 5, 0]), False, both=True),
]

DT = 1e-4   # depth_tol, epa_test.cpp:17
MT = 0.15   # mesh_tol, epa_test.cpp:19
ST = 0.05   # sym_tol, epa_test.cpp:21


def epa(line, a, b, depth=None, tol=DT, axis=None, mtv=False, positive=False,
        sym_depth_tol=None, normal_sum_max=None, both_depth=False):
    return {"src": f"{E}:{line}", "a": a, "b": b, "depth": depth, "tol": tol, "axis": axis,
            "mtv": mtv, "positive": positive, "sym_depth_tol": sym_depth_tol,
            "normal_sum_max": normal_sum_max, "both_depth": both_depth}


EPA = [
    epa(57, aabb(*U), aabb([0.5, -1, -1], [2.5, 1, 1]), 0.5),
    epa(69, aabb(*U), aabb([-1, 0.5, -1], [1, 2.5, 1]), 0.5),
    epa(80, aabb(*U), aabb([-1, -1, 0.5], [1, 1, 2.5]), 0.5),
    epa(90, aabb(*U), aabb([0.9, -1, -1], [2.9, 1, 1]), 0.1),
    epa(101, aabb(*U), aabb([-0.5, -1, -1], [1.5, 1, 1]), 1.5),
    epa(113, aabb([-2] * 3, [2] * 3), aabb([-0.5] * 3, [0.5] * 3), 2.5),
    epa(126, aabb(*U), aabb(*U), 2.0),
    epa(136, aabb(*U), aabb([-0.5, -1, -1], [0.5, 1, 1]), 1.5),
    epa(148, aabb([0] * 3, [2] * 3), aabb([1] * 3, [3] * 3), 1.0),
    epa(164, aabb(*U), aabb([0.5, -1, -1], [2.5, 1, 1]), axis=0),
    epa(176, aabb(*U), aabb([-1, 0.5, -1], [1, 2.5, 1]), axis=1),
    epa(187, aabb(*U), aabb([-1, -1, 0.5], [1, 1, 2.5]), axis=2),
    epa(198, aabb(*U), aabb([0.5, 0.3, -0.2], [2.5, 2.3, 1.8])),
    epa(211, aabb(*U), aabb([0.5, -1, -1], [2.5, 1, 1]), mtv=True),
    epa(220, aabb([0] * 3, [2] * 3), aabb([1] * 3, [3] * 3), mtv=True),
    epa(229, aabb([-3] * 3, [3] * 3), aabb(*U), mtv=True),
    epa(238, obb([0, 0, 0], I3), obb([1.5, 0, 0], I3), mtv=True),
    epa(247, obb([0, 0, 0], I3), obb([1, 0, 0], I3, Z45), mtv=True),
    epa(258, obb([0, 0, 0], (2, 0.2, 0.2)), obb([0, 0, 0], (2, 0.2, 0.2), Z90), mtv=True),
    epa(269, obb([0, 0, 0], I3), obb([1, 0.5, 0.3], I3, rot(PI / 6, (1, 1, 1))), mtv=True),
    epa(284, aabb(*U), aabb([0.5, -1, -1], [2.5, 1, 1]), sym_depth_tol=DT),
    epa(295, aabb(*U), aabb([0.5, -1, -1], [2.5, 1, 1]), normal_sum_max=0.1),
    epa(308, obb([0, 0, 0], I3), obb([1, 0, 0], I3, Z45), sym_depth_tol=ST),
    epa(322, obb([0, 0, 0], I3), obb([1, 0, 0], I3, Z45), normal_sum_max=0.3),
    epa(337, aabb([-3] * 3, [3] * 3), aabb(*U), sym_depth_tol=DT),
    epa(352, obb([0, 0, 0], I3), obb([1.5, 0, 0], I3), 0.5, axis=0),
    epa(364, obb([0, 0, 0], I3), obb([0, 0, 0], I3), 2.0),
    epa(373, obb([0, 0, 0], (2, 0.2, 0.2)), obb([0, 0, 0], (2, 0.2, 0.2), Z90), 0.4, tol=1e-2),
    epa(388, obb([0, 0, 0], I3), obb([1, 0, 0], I3, Z45), positive=True, mtv=True),
    epa(402, obb([0, 0, 0], (3, 0.3, 3)), obb([0, 0, 0], (0.3, 3, 0.3)), 3.3),
    epa(414, obb([0, 0, 0], I3), obb([0.5, 0.5, 0.5], I3, X90), positive=True, mtv=True),
    epa(431, obb([0, 0, 0], I3), aabb([0.5, -1, -1], [2.5, 1, 1]), 0.5, both_depth=True),
    epa(443, obb([0, 0, 0], (0.5, 0.5, 0.5)), aabb([-2] * 3, [2] * 3), 2.5),
    epa(459, box([0, 0, 0]), box([1.5, 0, 0]), 0.5),
    epa(471, box([0, 0, 0], (3, 3, 3)), box([0, 0, 0], (0.5, 0.5, 0.5)), 3.5),
    epa(485, box([0, 0, 0]), box([0, 0, 0]), 2.0),
    epa(495, box([0, 0, 0]), box([1.5, 0, 0]), axis=0),
    epa(505, box([0, 0, 0]), box([1.5, 0, 0]), sym_depth_tol=DT),
    epa(517, box([0, 0, 0]), box([1, 0, 0], r=Z45), positive=True, mtv=True),
    epa(535, sphere([0, 0, 0]), sphere([1.5, 0, 0]), 0.5, tol=MT),
    epa(547, sphere([0, 0, 0]), sphere([1.5, 0, 0]), axis=0),
    epa(557, sphere([0, 0, 0]), sphere([1, 1, 0]), 2.0 - math.sqrt(2.0), tol=MT),
    epa(571, box([0, 0, 0]), sphere([1.5, 0, 0]), 0.5, tol=MT),
    epa(588, pyramid([0, 0, 0]), pyramid([0, 1.5, 0]), positive=True),
    epa(599, pyramid([0, 0, 0]), pyramid([0, 1.5, 0]), mtv=True),
    epa(612, pyramid([0, 0, 0]), box([0, 0, 0]), positive=True, mtv=True),
    epa(628, pyramid([0, 0, 0]), pyramid([0, 3, 0], r=Z180), positive=True),
    epa(685, aabb(*U), aabb([0.99, -1, -1], [2.99, 1, 1]), 0.01, tol=1e-2),
    epa(697, aabb([-100] * 3, [100] * 3), aabb([-0.1] * 3, [0.1] * 3), 100.1, tol=0.5),
    epa(709, aabb([-3] * 3, [3] * 3), aabb([1] * 3, [2] * 3), 2.0),
    epa(721, obb([0, 0, 0], (5, 0.1, 5)), obb([0, 0.15, 0], (5, 0.1, 5)), 0.05, axis=1),
    epa(734, obb([0, 0, 0], I3), obb([0.5, 0.5, 0.5], I3, rot(PI / 3, (1, 2, 3))), positive=True, mtv=True),
    epa(747, box([0, 0, 0]), aabb([0.5, -1, -1], [2.5, 1, 1]), 0.5),
    epa(758, box([0, 0, 0]), obb([1.5, 0, 0], I3), 0.5),
]

# epa_depth_always_positive (epa_test.cpp:644-683): a unit box mesh against rotated/offset copies.
POSITIVE = [
    {"src": f"{E}:644", "a": box([0, 0, 0]), "b": box(p, r=r)}
    for p, r in [([1.5, 0, 0], None), ([0, 1.5, 0], None), ([0, 0, 1.5], None),
                 ([0.5, 0.5, 0.5], None), ([0, 0, 0], None), ([1.0, 0, 0], Z45),
                 ([0.3, 0.3, 0.3], rot(PI / 6, (1, 1, 1)))]
]

if __name__ == "__main__":
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "known_answers.json")
    with open(out, "w") as f:
        json.dump({"gjk": GJK, "epa": EPA, "epa_positive": POSITIVE,
                   "tolerances": {"depth_tol": DT, "mesh_tol": MT, "sym_tol": ST,
                                  "unit_normal": 1e-6, "mtv_nudge": 1e-3}}, f, indent=1)
    print(out, len(GJK), len(EPA), len(POSITIVE))
