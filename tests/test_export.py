"""The analysis export (src/visualization/enhanced_visualizer.py:1487-1560) on host arrays: file
names, JSON keys, the .npz arrays and the Reynolds number of calculate_flow_characteristics
(:450-471), with the reference's config scales (config/core.py:59-81, config/physics.py:42-111)."""
import json
import math

import numpy as np

from pour_over_coffee_lbm_gb300.diagnostics import export_data_for_analysis


class _Field:
    def __init__(self, a):
        self.a = a

    def to_numpy(self):
        return self.a.copy()


class _Lattice:
    def __init__(self, rho, u):
        self.NX, self.NY, self.NZ = rho.shape
        self.rho, self.u = _Field(rho), _Field(u)


class _Particles:
    def __init__(self, pos, vel, active):
        self.position, self.velocity, self.active = _Field(pos), _Field(vel), _Field(active)


class _Filter:
    def get_filter_statistics(self):
        return {"total_filter_nodes": 7, "average_resistance": 0.5, "average_blockage": 1.0,
                "average_flow_rate": 0.01, "max_blockage": 2.0}


def _case(seed=5):
    rng = np.random.default_rng(seed)
    shape = (6, 5, 4)
    rho = (1.0 + 0.01 * rng.normal(size=shape)).astype(np.float32)
    u = (0.01 * rng.normal(size=shape + (3,))).astype(np.float32)
    u[0] = 0.0
    return rho, u


def test_export_files_and_contents(tmp_path):
    rho, u = _case()
    pos = np.arange(12, dtype=np.float32).reshape(4, 3)
    vel = -pos
    active = np.array([1, 0, 1, 1], np.int32)
    out = export_data_for_analysis(_Lattice(rho, u), 1.5, 42, particles=_Particles(pos, vel, active),
                                   filter_system=_Filter(), out_dir=str(tmp_path))
    assert [p.split("/")[-1] for p in out] == ["cfd_data_export_step_0042.json", "cfd_data_export_step_0042.npz"]
    d = json.load(open(out[0]))
    assert set(d) == {"velocity_field", "density_field", "pressure_field", "particles", "filter", "metadata"}
    assert np.array_equal(np.array(d["velocity_field"]["u_y"], np.float32), u[..., 1])
    assert np.array_equal(np.array(d["velocity_field"]["magnitude"], np.float32),
                          np.sqrt(np.sum(u ** 2, axis=3)))
    assert d["particles"]["count"] == 3
    assert np.array_equal(np.array(d["particles"]["positions"], np.float32), pos[[0, 2, 3]])
    assert d["filter"]["total_filter_nodes"] == 7
    m = d["metadata"]
    assert m["simulation_time"] == 1.5 and m["step_number"] == 42 and m["grid_size"] == [6, 5, 4]
    assert math.isclose(m["physical_parameters"]["scale_length"], 0.000625)
    assert math.isclose(m["physical_parameters"]["scale_time"], 0.075)
    umag = np.sqrt(u[..., 0] ** 2 + u[..., 1] ** 2 + u[..., 2] ** 2) * 0.01
    re = float(np.mean(umag[umag > 1e-6])) * 0.085 / 3.15e-7
    assert math.isclose(m["physical_parameters"]["reynolds_number"], re, rel_tol=1e-12)
    z = np.load(out[1])
    # only the entries that are arrays go to the .npz, as float64 (NX, NY, NZ)
    assert sorted(z.files) == ["density_field", "pressure_field"]
    assert z["density_field"].dtype == np.float64 and z["density_field"].shape == rho.shape
    assert np.array_equal(z["density_field"], rho.astype(np.float64))
    assert np.array_equal(z["pressure_field"], (rho * np.float32(1.0 / 3.0)).astype(np.float64))


def test_export_at_rest_uses_the_characteristic_velocity(tmp_path):
    rho, u = _case()
    u[:] = 0.0
    out = export_data_for_analysis(_Lattice(rho, u), 0.0, 3, out_dir=str(tmp_path))
    d = json.load(open(out[0]))
    assert "particles" not in d and "filter" not in d
    assert math.isclose(d["metadata"]["physical_parameters"]["reynolds_number"], 0.02 * 0.085 / 3.15e-7)


def test_export_failure_returns_empty(tmp_path):
    rho, u = _case()
    assert export_data_for_analysis(_Lattice(rho, u), 0.0, 1, out_dir=str(tmp_path / "missing")) == []


def test_export_matches_the_reference_export(tmp_path):
    """The reference's own EnhancedVisualizer.export_data_for_analysis on the same inputs
    (tests/golden/export_reference.*, made by tests/golden/make_export_golden.py): file names,
    the JSON document and the .npz arrays, identical."""
    import os
    root = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    ref = json.load(open(os.path.join(root, "export_reference.json")))
    z = np.load(os.path.join(root, "export_reference.npz"))
    lat = _Lattice(z["rho"], z["u"])
    ps = _Particles(z["position"], z["velocity"], z["active"])

    class _RefFilter:
        def get_filter_statistics(self):
            return {"total_filter_nodes": 3, "average_resistance": 0.5, "average_blockage": 1.25,
                    "average_flow_rate": 0.002, "max_blockage": 4.0}

    out = export_data_for_analysis(lat, ref["simulation_time"], ref["step"], particles=ps,
                                   filter_system=_RefFilter(), out_dir=str(tmp_path))
    assert [p.split("/")[-1] for p in out] == ref["files"]
    assert json.load(open(out[0])) == ref["json"]
    ours = np.load(out[1])
    assert sorted(ours.files) == sorted(k[4:] for k in z.files if k.startswith("npz_"))
    for k in ours.files:
        assert ours[k].dtype == z["npz_" + k].dtype and np.array_equal(ours[k], z["npz_" + k]), k
