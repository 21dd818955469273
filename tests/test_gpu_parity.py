"""Parity of the CUDA FP64 path against the CPU oracle (through the C ABI).

Tolerances: particle counts and cell-sort indices bit-exact;
positions and momenta bit-exact after a push from identical state (the FP64
kernels are built without FMA contraction); per-mode fields and currents
within 1e-10 relative L2, the slack being the order of the FP64 atomic
current adds.

The oracle takes theta with libm's atan2, as the reference does, in the
single-push tests; the multi-step tests use its "shared" mode, the correctly
rounded atan2 that the kernel evaluates, because libm's last-bit errors (on
about 0.09 % of arguments) reach J_theta through the (m dtheta)^-2 deposit
factors and the thermal plasma's noise grows them past 1e-10 within tens of
steps (tests/test_gpu_math.py, test_libm_oracle_*).
"""
import numpy as np
import pytest

import cylindrical_epoch_gb300 as cg
from cylindrical_epoch_gb300 import abi
from tests.helpers import match_by_id, random_fields, rel_l2

pytestmark = pytest.mark.gpu

TOL_FIELD = 1.0e-10


def _pair(deck, fields=None, initialise=True, atan2="shared"):
    from oracle.oracle import Oracle
    parts, rng = cg.host_load(deck)
    gpu = cg.Run(deck, particles=parts, rng=rng, fields=fields, initialise=False)
    orc = Oracle(deck, particles=parts, rng=rng, atan2=atan2)
    if fields:
        for k, v in fields.items():
            orc.set_field(k, v)
    if initialise:
        gpu.lib.cyl_initialise(gpu.h)
        orc.initialise()
    return gpu, orc


def _cmp_fields(gpu, orc, names, tol=TOL_FIELD):
    worst = {}
    for n in names:
        a, b = gpu.field(n), orc.field(n)
        for m in range(a.shape[0]):
            if np.all(b[m] == 0) and np.all(a[m] == 0):
                continue
            e = rel_l2(a[m], b[m])
            worst[f"{n}[m={m}]"] = e
            assert e < tol, f"{n} mode {m}: rel L2 {e:.3e}"
    return worst


def test_push_bit_exact_positions(gpu_lib):
    deck = cg.thermal_plasma(nx=48, ny=24, ppc=6)
    flds = random_fields(deck, 1)
    gpu, orc = _pair(deck, fields=flds, initialise=False, atan2="libm")
    gpu.push_only()
    orc.stage("push")
    a, b = match_by_id(gpu.particles(0), orc.particles(0))
    for k in ("x", "y", "z", "px", "py", "pz", "w"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    _cmp_fields(gpu, orc, ["jxm", "jrm", "jtm"])


def test_cell_indices_after_push(gpu_lib):
    deck = cg.thermal_plasma(nx=40, ny=20, ppc=5)
    flds = random_fields(deck, 2)
    gpu, orc = _pair(deck, fields=flds, initialise=False, atan2="libm")
    gpu.push_only()
    orc.stage("push")
    ga = gpu.particles(0)
    gx, gy = gpu.cell_indices(0)
    ox, oy = orc.cell_indices(0)
    ob = orc.particles(0)
    og = np.argsort(ga.id)
    oo = np.argsort(ob.id)
    assert np.array_equal(gx[og], ox[oo])
    assert np.array_equal(gy[og], oy[oo])


def test_thermal_steps_parity(gpu_lib):
    deck = cg.thermal_plasma(nx=64, ny=32, ppc=8)
    gpu, orc = _pair(deck)
    gpu.step(1)
    orc.step(1)
    a, b = match_by_id(gpu.particles(0), orc.particles(0))
    for k in ("x", "y", "z", "px", "py", "pz"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), f"step 1 {k}"
    gpu.step(9)
    orc.step(9)
    sg, so = gpu.state(), orc.state()
    assert sg.n_live[0] == so.n_live[0]
    a, b = match_by_id(gpu.particles(0), orc.particles(0))
    for k in ("x", "y", "z"):
        assert rel_l2(getattr(a, k), getattr(b, k)) < 1e-12
    _cmp_fields_noisy(gpu, orc, deck, 10, ["exm", "erm", "etm", "bxm", "brm", "btm", "jxm", "jrm", "jtm"])


def _cmp_fields_noisy(gpu, orc, deck, nsteps, names):
    """Fields of a thermal-noise run after nsteps steps from t = 0.  Mode 0
    within 1e-10.  Modes m >= 1 of a thermal plasma amplify a last-bit change
    of a particle's angle through the deposit's (m dtheta)^-2 factors
    (particles.F90:603-625), and the device's atomic current additions
    change last bits of the fields from step 2 on.  The bar for m >= 1 is
    therefore the oracle's own response to last-bit angle changes: the same
    oracle with libm atan2, which differs from the correctly rounded one by
    one ulp on about 0.1 % of the angles (or 1e-10, if larger)."""
    from oracle.oracle import Oracle
    parts, rng = cg.host_load(deck)
    ulp = Oracle(deck, particles=parts, rng=rng, atan2="libm")
    ulp.initialise()
    ulp.step(nsteps)
    for n in names:
        g, o, u = gpu.field(n), orc.field(n), ulp.field(n)
        if np.all(o == 0) and np.all(g == 0):
            continue
        e0 = rel_l2(g[0], o[0])
        assert e0 < TOL_FIELD, f"{n} mode 0: rel L2 {e0:.3e}"
        for m in range(1, g.shape[0]):
            if np.all(o[m] == 0) and np.all(g[m] == 0):
                continue
            e, s = rel_l2(g[m], o[m]), rel_l2(u[m], o[m])
            assert e < max(TOL_FIELD, s), f"{n} mode {m}: rel L2 {e:.3e}, one-ulp response {s:.3e}"


def _small_wake(nsteps=80):
    deck = cg.wakefield(nx=128, ny=32, ppc=4, density=3.0e24, ramp=2.0e-6)
    # start the window early so that shifts happen inside a short test
    deck.window_start_time = 20 * 5.0e-17
    return deck


def test_wakefield_window_parity(gpu_lib):
    deck = _small_wake()
    gpu, orc = _pair(deck)
    for chunk in (1, 15, 24, 40):
        gpu.step(chunk)
        orc.step(chunk)
        sg, so = gpu.state(), orc.state()
        assert sg.step == so.step
        assert sg.n_shifts == so.n_shifts
        assert sg.x_grid_min == so.x_grid_min
        assert sg.n_live[0] == so.n_live[0], (sg.n_live[0], so.n_live[0])
    assert so.n_shifts > 10
    a, b = match_by_id(gpu.particles(0), orc.particles(0))
    for k in ("x", "y", "z"):
        assert rel_l2(getattr(a, k), getattr(b, k)) < 1e-12
    _cmp_fields(gpu, orc, ["exm", "erm", "etm", "bxm", "brm", "btm", "jxm", "jrm", "jtm"])


def test_graph_matches_eager(gpu_lib):
    deck = _small_wake()
    parts, rng = cg.host_load(deck)
    a = cg.Run(deck, particles=parts, rng=rng)
    b = cg.Run(deck, particles=parts, rng=rng)
    a.step(48, graph=False)
    b.step(48, graph=True)
    assert a.state().n_live[0] == b.state().n_live[0]
    for n in ("exm", "btm", "jxm"):
        assert rel_l2(b.field(n), a.field(n)) < 1e-10


def test_charge_density_and_continuity(gpu_lib):
    """cyl_charge_density against the oracle, and the discrete continuity
    residual of one step of the FP64 form: m = 0 at round-off, m = 1 equal
    to the oracle's (its theta current is not exactly conservative)."""
    from cylindrical_epoch_gb300.diagnostics import continuity_residual
    deck = cg.thermal_plasma(nx=64, ny=32, ppc=8)
    gpu, orc = _pair(deck)
    gpu.step(2)
    orc.step(2)
    r0g, r0o = gpu.charge_density(), orc.charge_density()
    for m in range(deck.n_mode):
        assert rel_l2(r0g[m], r0o[m]) < TOL_FIELD, m
    gpu.step(1)
    orc.step(1)
    r1g, r1o = gpu.charge_density(), orc.charge_density()
    dt = deck.grid_desc().dt
    rg = continuity_residual(deck, r0g, r1g, gpu.field("jxm"), gpu.field("jrm"), gpu.field("jtm"), dt)[0]
    ro = continuity_residual(deck, r0o, r1o, orc.field("jxm"), orc.field("jrm"), orc.field("jtm"), dt)[0]
    print("continuity residual per mode: gpu", rg, "oracle", ro)
    assert rg[0] < 1e-12
    assert abs(rg[1] - ro[1]) < 1e-8


def test_wide_window_shift(gpu_lib):
    """Window shifts on a grid 3200 cells long (a 3210-cell row of complex
    FP64 is 51 KB): counts, shifts and fields against the oracle."""
    deck = cg.wakefield(nx=3200, ny=16, ppc=1, density=3.0e24, ramp=2.0e-6)
    deck.window_start_time = 10 * 5.0e-17
    gpu, orc = _pair(deck)
    for chunk in (16, 24):
        gpu.step(chunk)
        orc.step(chunk)
        sg, so = gpu.state(), orc.state()
        assert sg.n_shifts == so.n_shifts and sg.n_live[0] == so.n_live[0]
    assert so.n_shifts > 10
    _cmp_fields(gpu, orc, ["exm", "erm", "btm", "jxm"])


def test_number_density_parity(gpu_lib):
    """cyl_number_density (calc_number_density_modes) against the oracle
    after a windowed laser-wakefield run, per mode, all species and one
    species."""
    deck = _small_wake()
    gpu, orc = _pair(deck)
    gpu.step(48)
    orc.step(48)
    assert orc.state().n_shifts > 0
    for isp in (-1, 0):
        a, b = gpu.number_density(isp), orc.number_density(isp)
        for m in range(deck.n_mode):
            assert rel_l2(a[m], b[m]) < TOL_FIELD, (isp, m)


def _steps_parity(deck, nsteps=10, fields=("exm", "erm", "etm", "bxm", "brm", "btm", "jxm", "jrm", "jtm")):
    gpu, orc = _pair(deck)
    gpu.step(1)
    orc.step(1)
    for isp in range(len(deck.species)):
        a, b = match_by_id(gpu.particles(isp), orc.particles(isp))
        for k in ("x", "y", "z", "px", "py", "pz"):
            assert np.array_equal(getattr(a, k), getattr(b, k)), (isp, k)
    gpu.step(nsteps - 1)
    orc.step(nsteps - 1)
    sg, so = gpu.state(), orc.state()
    for isp in range(len(deck.species)):
        assert sg.n_live[isp] == so.n_live[isp], isp
    _cmp_fields_noisy(gpu, orc, deck, nsteps, list(fields))
    return gpu, orc


@pytest.mark.parametrize("n_mode", [3, 4])
def test_more_modes_parity(gpu_lib, n_mode):
    """Modes m = 0..2 and 0..3 (the scan decks and the large deck)."""
    _steps_parity(cg.thermal_plasma(nx=48, ny=24, ppc=4, n_mode=n_mode))


def test_two_mobile_species_parity(gpu_lib):
    """Electrons and mobile thermal protons: both pushed, both deposit."""
    from cylindrical_epoch_gb300.deck import EV, KB, M0, Q0, Species
    deck = cg.thermal_plasma(nx=48, ny=24, ppc=4)
    t_k = 100.0 * EV / KB
    p = Species("proton", Q0, 1836.15267245 * M0, 2, 1.0e25, temp_k=(t_k, t_k, t_k), bc=deck.species[0].bc)
    p.capacity = 2 * deck.nx * deck.ny * 2 + 1024
    deck.species.append(p)
    _steps_parity(deck)


def test_reflecting_walls_parity(gpu_lib):
    """Reflecting particle walls and conducting field walls at both x ends
    (boundary.F90:1561-1569, the reflection folding of current_finish).  In
    16 steps about 1 % of the 1 keV electrons (v_th dt / dx = 0.027) cross a
    wall; longer runs let the order of the FP64 current additions move the
    noise-level m = 1 Bx past 1e-10."""
    deck = cg.thermal_plasma(nx=40, ny=20, ppc=6)
    walls = (abi.BC_REFLECT, abi.BC_REFLECT, abi.BC_OTHER, abi.BC_CONDUCT)
    deck.species[0].bc = walls
    deck.bc_field = (abi.BC_CONDUCT, abi.BC_CONDUCT, abi.BC_OTHER, abi.BC_CONDUCT)
    _steps_parity(deck, nsteps=16)


def test_current_smoothing_parity(gpu_lib):
    """smooth_mode_array (current_smooth.F90:145-196): two binomial passes and
    one compensation pass on a windowed laser wakefield."""
    deck = _small_wake()
    deck.smooth_currents, deck.smooth_its, deck.smooth_comp_its, deck.smooth_stride = 1, 2, 1, 1
    gpu, orc = _pair(deck)
    gpu.step(40)
    orc.step(40)
    assert gpu.state().n_live[0] == orc.state().n_live[0]
    assert orc.state().n_shifts > 0
    _cmp_fields(gpu, orc, ["exm", "erm", "btm", "jxm", "jrm", "jtm"])


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
def test_async_steps_and_pipelined_diagnostics(gpu_lib, precision):
    """cyl_step_async with each chunk's diagnostics read one chunk later
    (cyl_diagnostics_async / _read) gives, chunk by chunk, the diagnostics of
    synchronous steps and reads, and the same final state.  Energies within
    1e-10 relative in the FP64 form (the order of the FP64 atomic adds) and
    1e-6 in the mixed form, where that order also flips FP32 roundings of
    the stored fields (two identical mixed runs differ by about 1e-9)."""
    tol = 1e-10 if precision == abi.PREC_FP64 else 1e-6
    deck = cg.wakefield(nx=128, ny=32, ppc=4, density=3.0e24, ramp=2.0e-6, precision=precision)
    deck.window_start_time = 20 * 5.0e-17
    parts, rng = cg.host_load(deck)
    a = cg.Run(deck, particles=parts, rng=rng)
    b = cg.Run(deck, particles=parts, rng=rng)
    da, db = [], []
    for _ in range(5):
        a.step(16, graph=True)
        da.append(a.diagnostics())
    for i in range(5):
        b.step_async(16)
        if i:
            db.append(b.diagnostics_read())
        b.diagnostics_async()
    db.append(b.diagnostics_read())
    with pytest.raises(abi.CylError):
        b.diagnostics_read()  # nothing pending
    for x, y in zip(da, db):
        assert y.device_error == 0 and x.n_live == y.n_live
        for k in ("kinetic_energy", "field_energy_e", "field_energy_b"):
            assert abs(getattr(y, k) - getattr(x, k)) <= tol * abs(getattr(x, k)), k
    assert a.state().n_shifts == b.state().n_shifts > 10


@pytest.mark.parametrize("restart", [False, True])
def test_write_sdf_matches_fields(gpu_lib, tmp_path, restart):
    """cyl_write_sdf on a windowed run: every block holds the run's own
    downloaded mode array (rows of the Ex-staggered arrays shifted up by one,
    as the reference prints them), every species' particle blocks hold its
    downloaded live particles, the grid edges follow the moved window, and
    the header carries the run's step and time."""
    from oracle.sdf_read import read
    deck = _small_wake()
    run = cg.Run(deck)
    if restart:
        run.step_to_output(48)  # restart dumps are taken at the output point
    else:
        run.step(48, graph=True)
    p = tmp_path / "dump.sdf"
    run.write_sdf(p, restart=restart)
    h, inline, summary, data = read(p)
    s = run.state()
    assert h.step == s.step and h.time == s.time and h.restart_flag == int(restart)
    assert s.n_shifts > 0
    ng = abi.NG
    shifted = {"exm", "etm", "brm", "jxm", "jtm", "brm_old", "jxm_old", "jtm_old"}
    names = abi.FIELD_NAMES if restart else abi.FIELD_NAMES[:9]
    sp = [(s_.name, run.particles(i)) for i, s_ in enumerate(deck.species)]
    live = [(n_, p_) for n_, p_ in sp if p_.n > 0]
    nconst = (3 if s.window_started else 2) if restart else 0  # dt, window_shift_fraction, x_grid_min
    assert live and h.nblocks == nconst + 2 * len(names) + 6 * len(live) + 1
    if restart:
        assert data["dt"] == run.dt and data["x_grid_min"] == s.x_grid_min
        assert data.get("window_shift_fraction", 0.0) == (s.window_shift_fraction if s.window_started else 0.0)
    for n_, p_ in live:
        assert np.array_equal(data[f"grid/{n_}"], np.stack([p_.x, p_.y, p_.z]))
        for v, k in (("weight", "w"), ("px", "px"), ("py", "py"), ("pz", "pz"), ("id", "id")):
            assert np.array_equal(data[f"{v}/{n_}"], getattr(p_, k)), (v, n_)
    for name in names:
        a = run.field(name)
        sh = 1 if name in shifted else 0
        for part, v in (("real", a.real), ("imag", a.imag)):
            assert np.array_equal(data[f"{name}_{part}"], v[:, ng - sh:ng - sh + deck.ny, ng:ng + deck.nx]), name
    x, y = data["grid"]
    dx = (deck.x_max - deck.x_min) / deck.nx
    assert abs(x[0] - s.xb_min) <= 1e-15 * abs(s.xb_min) + 1e-30
    assert np.allclose(np.diff(x), dx, rtol=1e-12) and y[0] == 0.0


def test_libm_oracle_wakefield_window(gpu_lib):
    """The oracle with libm's atan2 (the reference's own call) against the
    device over 40 windowed laser-wakefield steps: libm's last-bit errors
    stay below the 1e-10 field bar on this deck."""
    deck = _small_wake()
    gpu, orc = _pair(deck, atan2="libm")
    gpu.step(40)
    orc.step(40)
    sg, so = gpu.state(), orc.state()
    assert sg.n_shifts == so.n_shifts > 0 and sg.n_live[0] == so.n_live[0]
    _cmp_fields(gpu, orc, ["exm", "erm", "etm", "bxm", "brm", "btm", "jxm", "jrm", "jtm"])


def test_libm_oracle_thermal_plasma(gpu_lib):
    """The same on 20 steps of the 1 keV thermal plasma, whose noise-level
    m = 1 fields amplify libm's last-bit atan2 errors: measured up to 7e-9
    relative (J_theta, B_x; 2e-12 after one push), every m = 0 field within
    1e-12.
    This is the spread of the reference's own result between a libm and a
    correctly rounded atan2 (x86 and Arm glibc 2.39 agree with each other)."""
    deck = cg.thermal_plasma(nx=64, ny=32, ppc=8)
    gpu, orc = _pair(deck, atan2="libm")
    gpu.step(20)
    orc.step(20)
    assert gpu.state().n_live[0] == orc.state().n_live[0]
    w = _cmp_fields(gpu, orc, ["exm", "erm", "etm", "bxm", "brm", "btm", "jxm", "jrm", "jtm"], tol=1e-7)
    print("libm oracle, thermal 20 steps:", w)
    assert all(v < 1e-12 for k, v in w.items() if k.endswith("[m=0]"))
