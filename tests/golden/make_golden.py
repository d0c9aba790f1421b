"""Extracts the known-answer values of RobotecGPULidar's own tests into reference_values.json.

Reads the reference test sources as text (never compiles or runs them) and records the constants the
tests assert on, so the test-suite can check this implementation and the oracle against them on a
machine without the reference tree. Run: python tests/golden/make_golden.py /path/to/RobotecGPULidar
"""
import json
import os
import re
import sys


def main(ref: str) -> None:
    t = lambda p: open(os.path.join(ref, p)).read()
    dft = t("test/src/graph/DistanceFieldTest.cpp")
    m = re.search(r"INSTANTIATE_TEST_CASE_P\(DistanceFieldTests, DistanceFieldTest, ::testing::Values\(([^)]*)\)\)", dft)
    cube_z = [float(v.strip().rstrip("f")) for v in m.group(1).split(",")]
    eps_mul = float(re.search(r"EPSILON_MUL = ([0-9.E*\s-]+);", dft).group(1).replace(" ", "").split("*")[0]) * float(
        re.search(r"EPSILON_MUL = [0-9.]+ \* ([0-9Ee-]+);", dft).group(1))
    eps_noise = float(re.search(r"EPSILON_NOISE = ([0-9.]+);", dft).group(1))
    noise = {k: float(re.search(k + r" = ([0-9.]+);", dft).group(1)) for k in ("STD_DEV", "STD_DEV_PER_METER", "MEAN")}
    readme = t("test/src/apiReadmeExample.cpp")
    readme_z = float(re.search(r"ASSERT_FLOAT_EQ\(results\[0\]\.value\[2\], ([0-9.]+)f\)", readme).group(1))
    mat = t("test/src/testMat3x4f.cpp")
    mats = [[float(x) for x in g.split(",")] for g in re.findall(r"\.rc = \{([^}]*)\}", mat)]
    geo = t("test/include/helpers/geometryData.hpp")
    half_edge = float(re.search(r"CUBE_HALF_EDGE = ([0-9.]+);", geo).group(1))
    common = t("test/include/helpers/commonHelpers.hpp")
    counts = int(re.search(r"maxGPUCoresTestCount = ([0-9]+);", common).group(1))
    comp = t("test/src/graph/nodes/CompactByFieldPointsNodeTest.cpp")
    chained = int(re.search(r"MULTIPLE_COMPACTIONS_COUNT = ([0-9]+);", comp).group(1))
    out = {
        "source": "RobotecGPULidar test sources (DistanceFieldTest.cpp, apiReadmeExample.cpp, testMat3x4f.cpp, "
                  "geometryData.hpp, commonHelpers.hpp, CompactByFieldPointsNodeTest.cpp)",
        "distance_field_cube_z": cube_z,
        "distance_field_epsilon": eps_mul,
        "noise_epsilon": eps_noise,
        "distance_noise": {"mean": noise["MEAN"], "st_dev": noise["STD_DEV"], "st_dev_per_meter": noise["STD_DEV_PER_METER"]},
        "cube_half_edge": half_edge,
        "readme_hit_z": readme_z,
        "mat3x4_mul": {"lhs": mats[0], "rhs": mats[1], "gold": mats[2]},
        "point_counts": [1, 100, counts],
        "chained_compactions": chained,
    }
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_values.json")
    json.dump(out, open(path, "w"), indent=1)
    print(path)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path of the RobotecGPULidar source tree>")
    main(sys.argv[1])
