"""Write tests/golden/pour_reference.npz from the reference's own PrecisePouringSystem
(src/physics/precise_pouring.py).  Its kernel source runs in this container through
taichi_standin.py, serially and in float32.

    python tests/golden/make_pour_golden.py <path of the reference checkout>

The script runs only where the reference checkout exists (its path is the script's required first argument).  The fixture
travels with tests/test_pour_oracle.py.  The reference reads its grid from `config`, so
NX = NY = NZ = 24 are set before construction.  Its nozzle then has diameter 8 cells, stream top
z = 18 and velocity 0.05 lu/ts, which the fixture records.

The fixture holds four cases:
- force: apply_pouring_force into a zero body force with no solid cells, spiral pattern, flow
  1.3, dt 0.5 (the first call advances pour_time to 0.5).  Recorded with the nozzle position the
  kernel used.
- trajectory: pour_time advanced by 0.9 per step and _get_current_pour_position, for 60 steps
  (the first two statements of apply_pouring_force).  Spiral from (32, 30) with NX = NY = 64.
- phase: apply_gradual_phase_change on a seeded phi in [-1, 1], dt 0.5.
- impact: create_water_impact_force on three particles (max force 0.05, dt 1).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
N = 24
TRAJ_NXY = 64


def main():
    sys.path.insert(0, HERE)
    import taichi_standin
    ti = taichi_standin.install()
    sys.path.insert(0, sys.argv[1])
    import config  # the reference's config package
    config.NX, config.NY, config.NZ = N, N, N
    from src.physics.precise_pouring import PrecisePouringSystem
    out = {}

    # force
    p = PrecisePouringSystem()
    out["diameter"], out["ztop"], out["velocity"] = p.POUR_DIAMETER_GRID, p.POUR_HEIGHT, p.POUR_VELOCITY
    p.start_pouring(center_x=11.3, center_y=12.6, flow_rate=1.3, pattern="spiral")
    bf = ti.Vector.field(3, ti.f32, (N, N, N))
    solid = ti.field(ti.u8, (N, N, N))
    p.apply_pouring_force(bf, solid, 0.5)
    out["force"] = bf.to_numpy()  # (NX, NY, NZ, 3)
    out["force_pos"] = np.array(p._get_current_pour_position(), np.float32)
    out["force_time"] = np.float32(p.pour_time[None])

    # trajectory, on a 64 x 64 plane so that the spiral reaches the clamp only late
    config.NX, config.NY = TRAJ_NXY, TRAJ_NXY
    q = PrecisePouringSystem()
    q.start_pouring(center_x=32.0, center_y=30.0, flow_rate=1.0, pattern="spiral")
    traj = []
    for _ in range(60):
        q.pour_time[None] += np.float32(0.9)
        traj.append(q._get_current_pour_position())
    out["trajectory"] = np.array(traj, np.float32)
    config.NX, config.NY = N, N

    # phase
    r = PrecisePouringSystem()
    r.start_pouring(center_x=12.0, center_y=11.0, flow_rate=1.3, pattern="center")
    rng = np.random.default_rng(5)
    phi0 = rng.uniform(-1.0, 1.0, size=(N, N, N)).astype(np.float32)
    phi = ti.field(ti.f32, (N, N, N))
    phi.from_numpy(phi0)
    r.apply_gradual_phase_change(phi, solid, 0.5)
    out["phase_in"], out["phase_out"] = phi0, phi.to_numpy()

    # impact
    s = PrecisePouringSystem()
    s.start_pouring(center_x=12.0, center_y=12.0, flow_rate=1.3, pattern="center")

    class Particles:
        pass
    ps = Particles()
    ps.particle_count = ti.field(ti.i32, ())
    ps.particle_count[None] = 3
    ps.active = ti.field(ti.i32, (3,))
    ps.active.from_numpy(np.ones(3, np.int32))
    ps.position = ti.Vector.field(3, ti.f32, (3,))
    ps.position.from_numpy(np.array([[12.7, 14.0, 12.0], [12.4, 12.0, 12.0], [16.0, 16.0, 5.0]], np.float32))
    ps.force = ti.Vector.field(3, ti.f32, (3,))
    s.create_water_impact_force(ps, 0.05, 1.0)
    out["impact_pos"], out["impact_force"] = ps.position.to_numpy(), ps.force.to_numpy()

    np.savez_compressed(os.path.join(HERE, "pour_reference.npz"), **out)
    print("wrote pour_reference.npz")


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: make_pour_golden.py <path of the reference checkout>")
    main()
