"""The committed fixtures under tests/golden/ are exactly what
tests/golden/make_golden.py extracts from the reference's test files: with
the maplab source tree named by MAPLAB_REFERENCE_ROOT, every fixture is
regenerated into a temporary directory and compared with the committed one.
Skipped where the source tree is absent."""
import importlib.util
import json
import os

import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
ROOT = os.environ.get("MAPLAB_REFERENCE_ROOT")
FIXTURES = ["imu_integrator.json", "reference_sensors.json", "error_term_scenarios.json",
            "pose_extrinsics_scenarios.json", "pose_parameterization_scenario.json", "camera_scenarios.json",
            "quaternion_math.json"]


@pytest.mark.skipif(not ROOT or not os.path.isdir(ROOT), reason="MAPLAB_REFERENCE_ROOT not set to a maplab tree")
def test_fixtures_regenerate_identically(tmp_path):
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    mg.main(ROOT, str(tmp_path))
    for name in FIXTURES:
        with open(os.path.join(GOLDEN, name)) as a, open(os.path.join(tmp_path, name)) as b:
            assert json.load(a) == json.load(b), name


def test_every_fixture_is_listed():
    present = sorted(f for f in os.listdir(GOLDEN) if f.endswith(".json"))
    assert present == sorted(FIXTURES)
