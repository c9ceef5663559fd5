"""Write tests/golden/export_reference.{json,npz}.  The fixture is the analysis export of the
reference's own EnhancedVisualizer (src/visualization/enhanced_visualizer.py:1487-1560), run on
seeded stub fields, plus the inputs it was given.

    python tests/golden/make_export_golden.py <path of the reference checkout>

The script runs only where the reference checkout exists (its path is the script's required first argument).  The fixture
travels with the tests (tests/test_export.py).

The visualiser module imports matplotlib at the top but does not use it on this path; an empty
stand-in module satisfies that import, since matplotlib is not installed here.

The export fails as shipped, for two reasons:
- calculate_flow_characteristics reads config.SCALE_DENSITY, which the reference's config does not
  define.  Here it is supplied as the 90 C water density, 965.3.  It feeds only a pressure
  statistic that the export does not write.
- With float32 fields, as Taichi's to_numpy() returns them, the Reynolds number is an np.float32
  that json cannot serialise.  The stub fields here are float64.
With those two inputs supplied, the reference writes both files, and they are stored as they are.
"""
import json
import os
import shutil
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SHAPE = (6, 5, 8)  # (NX, NY, NZ)


class _Stub(types.ModuleType):
    def __getattr__(self, k):
        if k.startswith("__"):
            raise AttributeError(k)
        m = _Stub(self.__name__ + "." + k)
        sys.modules[m.__name__] = m
        return m

    def __call__(self, *a, **k):
        return self


class Field:
    def __init__(self, a):
        self.a = a

    def to_numpy(self):
        return self.a.copy()


class Holder:
    pass


class Filter:
    def get_filter_statistics(self):
        return {"total_filter_nodes": 3, "average_resistance": 0.5, "average_blockage": 1.25,
                "average_flow_rate": 0.002, "max_blockage": 4.0}


def inputs(seed=7):
    rng = np.random.default_rng(seed)
    rho = 1.0 + 0.01 * rng.normal(size=SHAPE)
    u = 0.01 * rng.normal(size=SHAPE + (3,))
    u[:, :, 0] = 0.0  # a plane at rest (|u| below the 1e-6 m/s activity threshold)
    pos = rng.uniform(0, 5, size=(10, 3)).astype(np.float32)
    vel = rng.normal(size=(10, 3)).astype(np.float32)
    active = (rng.uniform(size=10) < 0.7).astype(np.int32)
    return rho, u, pos, vel, active


def main():
    sys.path.insert(0, sys.argv[1])
    for name in ("matplotlib", "matplotlib.pyplot", "matplotlib.colors", "matplotlib.patches", "matplotlib.gridspec"):
        sys.modules.setdefault(name, _Stub(name))
    import config  # the reference's config package
    config.SCALE_DENSITY = 965.3
    config.NX, config.NY, config.NZ = SHAPE
    from src.visualization.enhanced_visualizer import EnhancedVisualizer
    rho, u, pos, vel, active = inputs()
    lbm, ps = Holder(), Holder()
    lbm.rho, lbm.u = Field(rho), Field(u)
    ps.position, ps.velocity, ps.active = Field(pos), Field(vel), Field(active)
    work = tempfile.mkdtemp()
    cwd = os.getcwd()
    try:
        os.chdir(work)  # the visualiser writes its report folder and the export into the cwd
        viz = EnhancedVisualizer(lbm, None, None, ps, Filter())
        out = viz.export_data_for_analysis(12.5, 7)
        assert out, "the reference export failed"
        with open(out[0]) as f:
            exported = json.load(f)
        z = np.load(out[1])
        arrays = {k: z[k] for k in z.files}
    finally:
        os.chdir(cwd)
        shutil.rmtree(work)
    np.savez_compressed(os.path.join(HERE, "export_reference.npz"), rho=rho, u=u, position=pos, velocity=vel,
                        active=active, **{"npz_" + k: v for k, v in arrays.items()})
    with open(os.path.join(HERE, "export_reference.json"), "w") as f:
        json.dump({"simulation_time": 12.5, "step": 7, "files": [os.path.basename(p) for p in out],
                   "json": exported}, f)
    print("wrote export_reference.json / .npz")


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: make_export_golden.py <path of the reference checkout>")
    main()
