"""GPU parity of the particle rigid-body step.

Reference model: from identical state, one step must match the reference's
FP32 step within 1e-5 relative in position and velocity; the golden vectors
come from the reference's own kernels run on the host
(tests/golden/make_golden.py), so the bar here is the stricter bit-exact one
where the arithmetic allows it.  Config model: one GPU FP32 step against the
FP64 oracle, and the 100-step error reported."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5  # bound for one step against the reference FP32 step


def relerr(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-30)


def golden_rb(name="rb_ref_step_golden.npz"):
    return np.load(os.path.join(GOLDEN, name))


def golden_steps(g):
    return int(g["steps"]) if "steps" in g.files else 3


def make_ref_system(g, max_pairs=1 << 16):
    from gsap_gb300 import ParticleRigidBody
    s = {k[len("init__"):]: g[k].copy() for k in g.files if k.startswith("init__")}
    nb, np_ = len(s["pos"]), len(s["p_pos"])
    prb = ParticleRigidBody(nb, np_, max_pairs)
    prb.set_particle_data(s["ref_pos"], s["ref_mass"])
    prb.set_particle_shape_inv_inertia(s["shape_inv_inertia"])
    prb.set_rb_data(s)
    dt, spM, dpM, vmax, gy = (float(x) for x in g["params"])
    prb.set_params(spM, dpM)
    prb.set_contact(max_lin_vel=vmax, gravity_y=gy, floor_clamp=1, torque_quirk=1, pair_loop_quirk=1)
    return prb, s, dt


@pytest.mark.parametrize("fixture", ["rb_ref_step_golden.npz", "rb_demo_steps_golden.npz"])
@pytest.mark.parametrize("fused", [False, True])
def test_reference_step_matches_reference_kernels(cuda, fused, fixture):
    """A 64-body ring scene for 3 steps and the headless demo's scene (two
    hexagon sizes, 256 bodies in contact) for 4 steps, through the fused
    step and through the separate entry points in the demo's order."""
    from gsap_gb300 import MODE_SPHERE, Sap
    import oracle
    g = golden_rb(fixture)
    prb, s, dt = make_ref_system(g)
    sap = Sap(len(s["p_pos"]), mode=MODE_SPHERE)
    last = golden_steps(g) - 1
    for step in range(last + 1):
        if fused:
            prb.step(sap, dt)
        else:
            # the demo's order (demoParticles.h:875-912) through the separate entry points
            import torch
            prb.integrate(dt)
            prb.update_particle_data()
            pos = torch.from_numpy(prb.get_particles()["p_pos"]).to(cuda)
            pairs = torch.empty((1 << 16, 2), dtype=torch.int32, device=cuda)
            ent = torch.empty(len(s["p_pos"]) + 1, dtype=torch.int32, device=cuda)
            n_pairs, n_ent = sap.collision(0.0, pos, pairs, ent)
            prb.copy_in(3, pairs[:n_pairs].cpu().numpy())
            prb.copy_in(4, ent[:n_ent].cpu().numpy())
            prb.set_num_pairs(n_pairs, n_ent)
            assert n_pairs == int(g[f"step{step}__npairs"])
            prb.prepare()
            prb.compute_forces(dt)
            prb.update_velocity(dt)
        st = prb.get_state()
        pt = prb.get_particles()
        for k in ("pos", "quat", "lin_vel", "ang_vel"):
            want = g[f"step{step}__{k}"]
            assert relerr(st[k], want) <= REL_TOL, (step, k, relerr(st[k], want))
        for k in ("p_pos", "p_vel", "p_force"):
            want = g[f"step{step}__{k}"]
            assert relerr(pt[k], want) <= REL_TOL, (step, k, relerr(pt[k], want))
    sap.check()
    # the -fmad=false reference kernels reproduce the host-compiled
    # reference kernels exactly
    assert np.array_equal(st["pos"], g[f"step{last}__pos"])
    assert np.array_equal(st["lin_vel"], g[f"step{last}__lin_vel"])


def test_collision_matches_reference_format(cuda, oracle_lib):
    """Sap::collision drop-in: both-direction sorted int2 list and
    pairEntries equal to the oracle's format on the demo's particle layout."""
    import torch
    from gsap_gb300 import MODE_SPHERE, Sap
    rng = np.random.default_rng(11)
    for n in (24576, 5000, 2):
        c = rng.uniform(-12, 12, (n, 3)).astype(np.float32)
        c[:, 1] = np.abs(c[:, 1]) * 0.3
        s = np.concatenate([c, np.full((n, 1), 0.25, np.float32)], 1)
        sap = Sap(n, mode=MODE_SPHERE)
        pairs = torch.empty((max(16, 40 * n), 2), dtype=torch.int32, device=cuda)
        ent = torch.empty(n + 1, dtype=torch.int32, device=cuda)
        n_pairs, n_ent = sap.collision(0.0, torch.from_numpy(s).to(cuda), pairs, ent)
        want_pairs, want_ent = oracle_lib.both_directions(oracle_lib.bf_sphere(s))
        assert n_pairs == len(want_pairs) and n_ent == len(want_ent)
        assert np.array_equal(pairs[:n_pairs].cpu().numpy(), want_pairs)
        assert np.array_equal(ent[:n_ent].cpu().numpy(), want_ent)


def test_collision_format_with_long_rows(cuda, oracle_lib):
    """Both-direction format where rows are longer than the row buckets:
    a clump of 150 coincident spheres (rows of 149 entries each way) and a
    large sphere overlapping 1500 small ones (a row past the warp-sort
    limit), beside a scattered background."""
    import torch
    from gsap_gb300 import MODE_SPHERE, Sap
    rng = np.random.default_rng(23)
    bg = rng.uniform(-40, 40, (3000, 3)).astype(np.float32)
    clump = np.tile(np.float32([[30.0, 30.0, 30.0]]), (150, 1))
    ring = rng.uniform(-3, 3, (1500, 3)).astype(np.float32)
    c = np.concatenate([ring[:1], bg, clump, ring], 0)
    r = np.full((len(c), 1), 0.25, np.float32)
    r[0] = 6.0  # the large sphere, id 0
    s = np.concatenate([c, r], 1)
    n = len(s)
    sap = Sap(n, mode=MODE_SPHERE, pair_factor=64)
    pairs = torch.empty((64 * n, 2), dtype=torch.int32, device=cuda)
    ent = torch.empty(n + 1, dtype=torch.int32, device=cuda)
    n_pairs, n_ent = sap.collision(0.0, torch.from_numpy(s).to(cuda), pairs, ent)
    want_pairs, want_ent = oracle_lib.both_directions(oracle_lib.bf_sphere(s))
    assert n_pairs == len(want_pairs) and n_ent == len(want_ent)
    assert np.array_equal(pairs[:n_pairs].cpu().numpy(), want_pairs)
    assert np.array_equal(ent[:n_ent].cpu().numpy(), want_ent)


def config_params():
    return dict(dt=1.0 / 600.0, k=2e4, eta=50.0, kt=0.1, gravity_y=-9.81, box_lo=(0.0, 0.0, 0.0),
                box_hi=(200.0, 200.0, 200.0))


def make_cfg_system(sc, p, scenes_off=None):
    from gsap_gb300 import CONTACT_CONFIG, ParticleRigidBody, Sap
    nb, np_ = len(sc["pos"]), sc["n_particles"]
    prb = ParticleRigidBody(nb, np_, 16)
    prb.load_scene(sc)
    prb.set_contact(model=CONTACT_CONFIG, k=p["k"], eta=p["eta"], kt=p["kt"], gravity_y=p["gravity_y"],
                    box_lo=p["box_lo"], box_hi=p["box_hi"])
    S = 1 if scenes_off is None else len(scenes_off) - 1
    if scenes_off is not None:
        prb.set_scenes(scenes_off)
    sap = Sap(nb, max_scenes=S)
    return prb, sap


# Free-running 100-step trajectory error against the FP64 oracle.  The
# trajectory is chaotic once bodies collide (a contact that starts one step
# earlier on one side changes everything after it), so this bounds drift,
# not rounding: measured on a GB300 at pos 3.7e-4 / 7.1e-4 and velocity
# 8.6e-3 / 1.5e-2 for the two scenes below, asserted with margin.
FREE_RUN_TOL = {"pos": 3e-3, "lin_vel": 5e-2}
# At most this share of the bodies may be left out of a step's comparison
# for a contact at the onset threshold (see oracle/trajectory.py).
LEFT_OUT_SHARE = 0.01


def check_fp64_errors(e, nb):
    print("per-step max", e["per_step_max"], "all bodies", e["per_step_max_all_bodies"],
          "left out (max, mean)", e["bodies_left_out_max"], e["bodies_left_out_mean"],
          "free-running", e["free_running"])
    assert e["per_step_max"]["pos"] <= REL_TOL
    assert e["per_step_max"]["lin_vel"] <= REL_TOL
    assert e["per_step_max"]["ang_vel"] <= REL_TOL
    assert e["bodies_left_out_max"] <= LEFT_OUT_SHARE * nb
    for k, tol in FREE_RUN_TOL.items():
        assert e["free_running"][k] <= tol, (k, e["free_running"][k])


def test_config_steps_vs_fp64_oracle(cuda, oracle_lib):
    """Dense 2048-cube scene (the 65,536-cube workload's model, k=2e4,
    damping 50, tangential 0.1, dt=1/600): every one of 100 steps, taken
    from the FP64 oracle's state, within 1e-5 relative of the oracle's next
    state in position and velocity (bodies with a contact at the onset
    threshold left out and counted); the free-running trajectory bounded."""
    from oracle.trajectory import fp64_errors
    from gsap_gb300 import scenes
    p = config_params()
    sc = scenes.cubes_in_box(2048, box=40.0, seed=1)  # dense: many contacts
    p["box_hi"] = (40.0, 40.0, 40.0)
    prb, sap = make_cfg_system(sc, p)
    check_fp64_errors(fp64_errors(prb, sap, sc, p, steps=100), 2048)


def test_batched_config_steps_vs_fp64_oracle(cuda, oracle_lib):
    """Batched form of the same check (the 1024-scene workload's shapes:
    cubes, rods and L shapes; scene sizes log-uniform): 16 scenes of 64 to
    1024 bodies stepped in one batch, every step from the oracle's state
    within 1e-5, and the oracle run on the first 8 scenes only must agree
    with the batch there (scenes never interact)."""
    from oracle.trajectory import fp64_errors
    from gsap_gb300 import scenes
    p = config_params()
    p["box_hi"] = (30.0, 30.0, 30.0)
    sc = scenes.mixed_scenes(S=16, seed=5, lo=64, hi=1024, box=30.0)
    prb, sap = make_cfg_system(sc, p, sc["body_offsets"])
    check_fp64_errors(fp64_errors(prb, sap, sc, p, steps=100), len(sc["pos"]))
    part = fp64_errors(prb, sap, sc, p, steps=20, check_scenes=8)
    assert part["checked_bodies"] == int(sc["body_offsets"][8])
    assert part["per_step_max"]["pos"] <= REL_TOL and part["per_step_max"]["lin_vel"] <= REL_TOL


def test_headless_demo_runs_and_restarts_from_snapshot(cuda, tmp_path):
    """The DemoParticles scene stepped headless; a run restarted from a
    binary snapshot continues like the uninterrupted one."""
    from gsap_gb300 import demo
    sc = demo.demo_scene(512, n_row=8, seed=1)
    d = demo.Demo(sc)
    d.run(30)
    st = d.state()
    assert all(np.isfinite(st[k]).all() for k in st)
    assert st["pos"][:, 1].mean() < sc["pos"][:, 1].mean() - 0.5  # falling under gravity
    path = tmp_path / "snap.npz"
    demo.save_snapshot(path, sc, st, d.steps)
    d.run(10)
    a = d.state()
    d.sap.check()
    sc2, step = demo.load_snapshot(path)
    assert step == 30
    d2 = demo.Demo(sc2)
    d2.run(10)
    b = d2.state()
    for k in ("pos", "lin_vel"):
        assert relerr(b[k][:, :3], a[k][:, :3]) < 1e-4, k


def test_prbwrap_launchers_match_reference_kernels(cuda, oracle_lib):
    """The six gsap_k_* launchers (PRBWrap, ParticleRigidBodyWrapper.h:11-54)
    on caller-owned device arrays, in the demo's order
    (demoParticles.h:875-912) with the particle broadphase of
    gsap_sap_collision, reproduce the reference kernels' golden steps bit
    for bit."""
    import ctypes as C

    import torch
    from gsap_gb300 import MODE_SPHERE, Sap, _lib
    from gsap_gb300._lib import ContactParams, check
    L = _lib.load()
    g = golden_rb()
    s = {k[len("init__"):]: g[k].copy() for k in g.files if k.startswith("init__")}
    dt, spM, dpM, vmax, gy = (float(x) for x in g["params"])
    nb, np_ = len(s["pos"]), len(s["p_pos"])
    quat = oracle_lib.normalize_quats(np.ascontiguousarray(s["quat"], np.float32))  # setRbData's upload step

    def dev(a, dtype=torch.float32):
        return torch.from_numpy(np.ascontiguousarray(a)).to(cuda).view(dtype)

    d = {k: dev(s[k]) for k in ("pos", "lin_vel", "ang_vel", "inv_mass", "inv_inertia", "ref_pos", "ref_mass",
                                "shape_inv_inertia", "p_pos", "p_vel", "p_force", "p_mass")}
    d["quat"] = dev(quat)
    for k in ("shape_idx", "p_start", "n_part"):
        d[k] = dev(s[k].astype(np.int32), torch.int32)
    cp = ContactParams()
    cp.model, cp.gravity_y, cp.floor_clamp = 0, gy, 1
    sap = Sap(np_, mode=MODE_SPHERE)
    pairs = torch.empty((1 << 16, 2), dtype=torch.int32, device=cuda)
    ent = torch.empty(np_ + 1, dtype=torch.int32, device=cuda)
    ptr = {k: v.data_ptr() for k, v in d.items()}
    for step in range(golden_steps(g)):
        check(L.gsap_k_integrate(ptr["pos"], ptr["quat"], ptr["lin_vel"], ptr["ang_vel"], C.c_float(dt), nb,
                                 C.byref(cp), None))
        check(L.gsap_k_update_particle_data(ptr["pos"], ptr["quat"], ptr["lin_vel"], ptr["ang_vel"],
                                            ptr["shape_idx"], ptr["p_start"], ptr["n_part"], ptr["ref_pos"],
                                            ptr["ref_mass"], ptr["p_pos"], ptr["p_vel"], ptr["p_mass"], nb, None))
        n_pairs, n_ent = sap.collision(0.0, d["p_pos"].view(np_, 4), pairs, ent)
        assert n_pairs == int(g[f"step{step}__npairs"])
        check(L.gsap_k_prepare(ptr["quat"], ptr["shape_idx"], ptr["shape_inv_inertia"], ptr["inv_inertia"], nb, None))
        check(L.gsap_k_clear_force_and_boundary(ptr["p_pos"], ptr["p_vel"], ptr["p_mass"], ptr["p_force"],
                                                C.c_float(spM), C.c_float(dpM), np_, C.c_float(dt), None))
        check(L.gsap_k_compute_force_on_particles(ptr["p_pos"], ptr["p_vel"], pairs.data_ptr(), ent.data_ptr(),
                                                  n_pairs, n_ent, ptr["p_mass"], C.c_float(spM), C.c_float(dpM),
                                                  ptr["p_force"], C.c_float(dt), 1, None))
        check(L.gsap_k_update_velocity(ptr["lin_vel"], ptr["ang_vel"], ptr["quat"], ptr["inv_mass"],
                                       ptr["inv_inertia"], ptr["shape_idx"], ptr["p_start"], ptr["n_part"],
                                       ptr["ref_pos"], ptr["p_force"], nb, C.c_float(dt), C.c_float(vmax),
                                       1 if vmax > 0 else 0, 1, None))
        torch.cuda.synchronize()
        for k in ("pos", "quat", "lin_vel", "ang_vel", "p_pos", "p_vel", "p_force"):
            got = d[k].cpu().numpy().reshape(g[f"step{step}__{k}"].shape)
            assert np.array_equal(got, g[f"step{step}__{k}"]), (step, k, relerr(got, g[f"step{step}__{k}"]))
        # prepare's world inverse inertia: the three matrix rows (the unused
        # w lane of the reference's float4 rows carries rounding residue)
        got = d["inv_inertia"].cpu().numpy().reshape(-1, 3, 4)[:, :, :3]
        assert np.array_equal(got, g[f"step{step}__inv_inertia"].reshape(-1, 3, 4)[:, :, :3]), step
