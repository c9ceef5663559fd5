"""z-slab decomposition, CPU: the halo protocol of pour_over_coffee_lbm_gb300.slabs between
processes (RankHalo over gloo, world size 2 and 3) drives a numpy AA stepper and must reproduce the
undivided run bit for bit, on a mask whose walls cross the slab interfaces (the masked copy-back
case) and with flow through them; plus the host-side helpers."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import np_aa
from pour_over_coffee_lbm_gb300.params import RED_COUNT
from pour_over_coffee_lbm_gb300.slabs import DOWN, UP, RankHalo, slab_bounds, slab_flags, writer_masks

NX, NY, NZ, STEPS, OMEGA = 14, 12, 18, 23, 1.25


def _case():
    rng = np.random.default_rng(5)
    solid = rng.uniform(size=(NZ, NY, NX)) < 0.12
    solid[0] = solid[-1] = True
    solid[:, 0] = solid[:, -1] = True
    solid[:, :, 0] = solid[:, :, -1] = True
    flags = np_aa.link_flags(solid)
    f = np.zeros((19, NZ, NY, NX))
    fluid = ~solid
    for q in range(19):
        f[q][fluid] = np_aa.W[q] * (1.0 + 0.05 * rng.uniform(-1, 1, size=int(fluid.sum())))
    return flags, f


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, outdir):
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    flags, f = _case()
    z0, z1 = slab_bounds(NZ, world)[rank]
    fl = slab_flags(flags, z0, z1)
    fs = np.zeros((19, z1 - z0 + 2, NY, NX))
    lo, hi = max(z0 - 1, 0), min(z1 + 1, NZ)
    fs[:, lo - (z0 - 1): hi - (z0 - 1)] = f[:, lo:hi]
    ft = torch.from_numpy(fs)  # shares memory with fs
    halo = RankHalo(fl, rank, world)
    for t in range(STEPS):
        if t % 2:
            halo.exchange_in(ft)
        np_aa.aa_step(fs, fl, t, OMEGA)
        if t % 2:
            halo.exchange_out(ft)
    if STEPS % 2:
        halo.exchange_in(ft)  # an odd-parity state is read through the ghost slots
    np.save(os.path.join(outdir, "slab%d.npy" % rank), fs)
    dist.barrier()
    dist.destroy_process_group()


def _natural(f, flags, t):
    """Natural-layout state of an AA buffer at time t (odd: the odd-step read gather)."""
    if t % 2 == 0:
        return f.copy()
    nz, ny, nx = flags.shape
    n = nz * ny * nx
    F = f.reshape(19, n)
    fl = flags.reshape(n).astype(np.int64)
    c = np.arange(n)
    lo = nx * ny + nx + 1
    live = ((fl & 1) == 0) & (c >= lo) & (c <= n - 1 - lo)
    out = np.zeros_like(F)
    cells, flc = c[live], fl[live]
    off = np_aa.CX + np_aa.CY * nx + np_aa.CZ * nx * ny
    for q in range(19):
        wall = (q != 0) & (((flc >> (8 + np_aa.OPP[q])) & 1) == 1)
        out[q, cells] = np.where(wall, F[q, cells], F[np_aa.OPP[q], cells - off[q]])
    return out.reshape(f.shape)


@pytest.mark.parametrize("world", [2, 3])
def test_rank_halo_matches_undivided(tmp_path, world):
    flags, f = _case()
    ref = f.copy()
    for t in range(STEPS):
        np_aa.aa_step(ref, flags, t, OMEGA)
    ref_nat = _natural(ref, flags, STEPS)
    mp.start_processes(_rank, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    got = np.zeros_like(f)
    for r, (z0, z1) in enumerate(slab_bounds(NZ, world)):
        fs = np.load(tmp_path / ("slab%d.npy" % r))
        nat = _natural(fs, slab_flags(flags, z0, z1), STEPS)
        got[:, z0:z1] = nat[:, 1:-1]
    live = np.zeros(flags.shape, bool)
    live[1:-1, 1:-1, 1:-1] = (flags[1:-1, 1:-1, 1:-1] & 1) == 0
    assert np.array_equal(got[:, live], ref_nat[:, live])
    assert np.abs(ref_nat[:, live] - f[:, live]).max() > 1e-3  # the state did evolve


def test_slab_helpers():
    assert UP == [5, 11, 12, 15, 16] and DOWN == [6, 13, 14, 17, 18]
    assert slab_bounds(10, 3) == [(0, 3), (3, 6), (6, 10)]
    with pytest.raises(ValueError):
        slab_bounds(4, 3)
    fl = np.arange(5 * 2 * 2, dtype=np.uint32).reshape(5, 2, 2) * 2  # even: no SOLID bit
    s = slab_flags(fl, 0, 2)
    assert (s[0] == 1).all() and np.array_equal(s[1:], fl[:3])
    s = slab_flags(fl, 3, 5)
    assert np.array_equal(s[:3], fl[2:5]) and (s[3] == 1).all()
    plane = np.zeros((4, 5), np.uint32)
    plane[1, 2] = 1  # one solid writer
    m = writer_masks(plane, DOWN)
    for a, q in enumerate(DOWN):
        cx, cy = int(np_aa.CX[q]), int(np_aa.CY[q])
        for j in range(4):
            for i in range(5):
                jj, ii = j - cy, i - cx
                inside = 0 <= jj < 4 and 0 <= ii < 5
                assert m[a, j, i] == (inside and not (jj == 1 and ii == 2))


# ---- the same protocol driving the oracle's restatement of the product's AA step -------------------
def _v60_case():
    from pour_over_coffee_lbm_gb300.params import LES_LOCAL, STORE_F64, LatticeConfig
    # a V60 lattice with flow through the slab interfaces: inlet jet, LES, porous band, gravity
    return LatticeConfig(nx=20, ny=18, nz=24, band_thickness=2.0, les_mode=LES_LOCAL, u_inlet=-0.05,
                         cs_smag=0.3, storage=STORE_F64)


ORC_STEPS = 17


def _rank_oracle(rank, world, port, outdir):
    import oracle
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    cfg = _v60_case()
    flags = oracle.build_flags(cfg)
    f = oracle.init_equilibrium(cfg, flags, np.float64)
    z0, z1 = slab_bounds(cfg.nz, world)[rank]
    fl = slab_flags(flags, z0, z1)
    fs = np.zeros((19, z1 - z0 + 2, cfg.ny, cfg.nx))
    lo, hi = max(z0 - 1, 0), min(z1 + 1, cfg.nz)
    fs[:, lo - (z0 - 1): hi - (z0 - 1)] = f[:, lo:hi]
    ft = torch.from_numpy(fs)  # shares memory with fs
    halo = RankHalo(fl, rank, world)
    scfg = cfg.replace(nz=z1 - z0 + 2)
    red = np.zeros(RED_COUNT)
    for t in range(ORC_STEPS):
        if t % 2:
            halo.exchange_in(ft)
        oracle.step_aa(scfg, fl, fs, t, reductions=red)
        if t % 2:
            halo.exchange_out(ft)
    if ORC_STEPS % 2:
        halo.exchange_in(ft)
    np.save(os.path.join(outdir, "oslab%d.npy" % rank), fs)
    # the step sums of the owned planes, and an integer count, summed over the ranks
    tot = halo.reduce_sums(torch.from_numpy(red))
    cnt = halo.reduce_sums(torch.tensor([int(((fl[1:-1] & 1) == 0).sum())], dtype=torch.int64))
    np.save(os.path.join(outdir, "ored%d.npy" % rank), np.concatenate([tot.numpy(), cnt.numpy().astype(np.float64)]))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_rank_halo_with_the_oracle_aa_step(tmp_path, world):
    """gloo ranks each step their z-slab with the oracle's AA step (the product's stepping order and
    collision) through RankHalo; the assembled state equals the undivided oracle AA run and the
    oracle's push run bit for bit."""
    import oracle
    cfg = _v60_case()
    flags = oracle.build_flags(cfg)
    f0 = oracle.init_equilibrium(cfg, flags, np.float64)
    aa = f0.copy()
    push = f0.copy()
    for t in range(ORC_STEPS):
        oracle.step_aa(cfg, flags, aa, t)
        push, _, _ = oracle.step(cfg, flags, push)
    ref = _natural(aa, flags, ORC_STEPS)
    fluid = (flags & 1) == 0
    inner = np.zeros(flags.shape, bool)
    inner[1:-1, 1:-1, 1:-1] = True
    live = fluid & inner
    assert np.array_equal(ref[:, live], push[:, live])  # AA order == push order, bit for bit
    mp.start_processes(_rank_oracle, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    got = np.zeros_like(f0)
    for r, (z0, z1) in enumerate(slab_bounds(cfg.nz, world)):
        fs = np.load(tmp_path / ("oslab%d.npy" % r))
        got[:, z0:z1] = _natural(fs, slab_flags(flags, z0, z1), ORC_STEPS)[:, 1:-1]
    assert np.array_equal(got[:, live], ref[:, live])
    assert np.abs(ref[:, live] - f0[:, live]).max() > 1e-4  # the state did evolve
    # all-reduced step sums: the undivided run's, up to the order of the FP64 additions
    red = np.zeros(RED_COUNT)
    aa = f0.copy()
    for t in range(ORC_STEPS):
        oracle.step_aa(cfg, flags, aa, t, reductions=red)
    for r in range(world):
        got_red = np.load(tmp_path / ("ored%d.npy" % r))
        assert np.allclose(got_red[:RED_COUNT], red, rtol=1e-12, atol=1e-12 * abs(red[0])), (got_red, red)
        assert got_red[RED_COUNT] == int(((flags[:, :, :] & 1) == 0).sum())


# ---- slab-owned particles (RankParticles) with the oracle's coupling pass and AA step --------------
P_STEPS = 10


def _coupled_slab_case():
    from pour_over_coffee_lbm_gb300.params import LES_LOCAL, LatticeConfig, ParticleConfig
    cfg = LatticeConfig(nx=20, ny=18, nz=28, band_thickness=2.0, les_mode=LES_LOCAL, u_inlet=-0.05, cs_smag=0.3)
    pc = ParticleConfig(count=600, deterministic=True, density_ratio=1.5)
    rng = np.random.default_rng(31)
    n = pc.count
    cx, cy = cfg.axis
    # particles around the interfaces z = 9 and z = 18 of three slabs, moving up or down across them
    zc = np.where(rng.uniform(size=n) < 0.5, 9.0, 18.0)
    z = zc + rng.uniform(-0.3, 0.3, n)
    r = 0.5 * (z - cfg.cone_apex_z) * np.tan(np.radians(cfg.cone_half_angle_deg)) * np.sqrt(rng.uniform(size=n))
    a = rng.uniform(0, 2 * np.pi, n)
    pos = np.stack([cx + r * np.cos(a), cy + r * np.sin(a), z]).astype(np.float32)
    vel = np.zeros((3, n), np.float32)
    vel[2] = rng.choice([-0.15, 0.15], n).astype(np.float32)
    d = np.exp(rng.normal(np.log(0.6), 0.3, n)).astype(np.float32)
    act = np.ones(n, np.int32)
    return cfg, pc, pos, vel, d, act


def _rank_particles(rank, world, port, outdir):
    import oracle
    from pour_over_coffee_lbm_gb300.slabs import RankParticles, owner_plane
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    cfg, pc, pos, vel, d, act = _coupled_slab_case()
    nz, ny, nx = cfg.nz, cfg.ny, cfg.nx
    flags = oracle.build_flags(cfg)
    z0, z1 = slab_bounds(nz, world)[rank]
    fl = slab_flags(flags, z0, z1)
    nzs = z1 - z0 + 2
    scfg = cfg.replace(nz=nzs)
    f = oracle.init_equilibrium(cfg, flags, np.float32)
    fs = np.zeros((19, nzs, ny, nx), np.float32)
    lo, hi = max(z0 - 1, 0), min(z1 + 1, nz)
    fs[:, lo - (z0 - 1): hi - (z0 - 1)] = f[:, lo:hi]
    ft = torch.from_numpy(fs)
    halo = RankHalo(fl, rank, world)
    rp = RankParticles(rank, world, z0, z1, nz)
    k = owner_plane(torch.from_numpy(pos[2]), nz)
    mine = ((k >= z0) & (k < z1)).numpy()
    parts = {"pos": torch.from_numpy(pos[:, mine].copy()), "vel": torch.from_numpy(vel[:, mine].copy()),
             "diam": torch.from_numpy(d[mine].copy()), "drag_old": torch.zeros((3, int(mine.sum())), dtype=torch.float32),
             "active": torch.from_numpy(act[mine].copy()), "ident": torch.arange(pc.count)[torch.from_numpy(mine)]}
    u = torch.zeros((3, nzs, ny, nx), dtype=torch.float32)
    moved = 0
    for t in range(P_STEPS):
        rp.exchange_u(u)
        ug = np.zeros((3, nz, ny, nx), np.float32)  # this slab's planes z0 - 1 .. z1 of the global u
        ug[:, lo:hi] = u.numpy()[:, lo - (z0 - 1): hi - (z0 - 1)]
        ppos, pvel, pdrag_old, pact, fix, _ = oracle.particles_couple(
            cfg, pc, parts["pos"].numpy(), parts["vel"].numpy(), parts["diam"].numpy(), parts["drag_old"].numpy(),
            parts["active"].numpy(), ug)
        fix = fix.reshape(4, nz, ny, nx)
        assert not fix[:, :z0].any() and not fix[:, z1 + 1:].any()  # corners stay within z0 .. z1
        dep = torch.zeros((4, nzs, ny, nx), dtype=torch.int64)
        dep[:, lo - (z0 - 1): hi - (z0 - 1)] = torch.from_numpy(fix[:, lo:hi])
        rp.reduce_deposit(dep)
        pdrag = (dep.double() / 2.0 ** 32).float().numpy()
        parts.update(pos=torch.from_numpy(ppos), vel=torch.from_numpy(pvel), drag_old=torch.from_numpy(pdrag_old),
                     active=torch.from_numpy(pact))
        before = parts["ident"].clone()
        parts = rp.migrate(parts)
        moved += int((~torch.isin(parts["ident"], before)).sum())
        if t % 2:
            halo.exchange_in(ft)
        _, un = oracle.step_aa(scfg, fl, fs, t, pdrag=pdrag, macro=True)
        if t % 2:
            halo.exchange_out(ft)
        u = torch.from_numpy(un)
    if P_STEPS % 2:
        halo.exchange_in(ft)
    np.savez(os.path.join(outdir, "pslab%d.npz" % rank), f=fs, moved=moved,
             **{k: v.numpy() for k, v in parts.items()})
    dist.barrier()
    dist.destroy_process_group()


def test_slab_owned_particles_match_undivided(tmp_path):
    """Three gloo ranks, particles owned by slab: the u ghost plane, the deposit's reduce-add and
    the migration across the interfaces reproduce the undivided coupled run bit for bit."""
    import oracle
    world = 3
    cfg, pc, pos, vel, d, act = _coupled_slab_case()
    flags = oracle.build_flags(cfg)
    f = oracle.init_equilibrium(cfg, flags, np.float32)
    u = np.zeros((3, cfg.nz, cfg.ny, cfg.nx), np.float32)
    drag = np.zeros_like(pos)
    for t in range(P_STEPS):
        pos, vel, drag, act, fix, _ = oracle.particles_couple(cfg, pc, pos, vel, d, drag, act, u)
        pdrag = (fix.astype(np.float64) / 2.0 ** 32).astype(np.float32).reshape(4, cfg.nz, cfg.ny, cfg.nx)
        _, u = oracle.step_aa(cfg, flags, f, t, pdrag=pdrag, macro=True)
    ref = _natural(f, flags, P_STEPS)
    mp.start_processes(_rank_particles, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    got = np.zeros_like(f)
    gpos = np.full_like(pos, np.nan)
    seen = np.zeros(pc.count, int)
    moved = 0
    for r, (z0, z1) in enumerate(slab_bounds(cfg.nz, world)):
        z = np.load(tmp_path / ("pslab%d.npz" % r))
        got[:, z0:z1] = _natural(z["f"], slab_flags(flags, z0, z1), P_STEPS)[:, 1:-1]
        gpos[:, z["ident"]] = z["pos"]
        seen[z["ident"]] += 1
        moved += int(z["moved"])
    live = np.zeros(flags.shape, bool)
    live[1:-1, 1:-1, 1:-1] = (flags[1:-1, 1:-1, 1:-1] & 1) == 0
    assert np.all(seen == 1)  # every particle owned by exactly one rank
    assert moved > 20  # particles did cross the interfaces
    assert np.array_equal(gpos, pos)
    assert np.array_equal(got[:, live], ref[:, live])
