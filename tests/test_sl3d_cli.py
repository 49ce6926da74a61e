"""The sl3d front end (sl3dpp_gb300/csrc/app/sl3d.cpp): the reference's
`sl3d solve` for a 3D run through time (apps/SolveCommand.cpp:1747-1795) with
its disk checkpoints (:239-290) and restart, and `sl3d kernel` (the
discrete adjoint's kernels of point and cap measurements, the run without an
ocean).

Without a GPU: configs are read and checked (`sl3d check`): unknown members,
bad values and missing blocks are refused; the run hash depends on the
members that decide the computation and not on the key order or on the
members that only steer the run. On the GPU: a run's surface table is the
library's own evolution (Evolution3D.Run through the C ABI) on the same
inputs, number for number; a run stopped after a node and restarted from its
checkpoint writes the uninterrupted run's table bit for bit; another run's
checkpoint is refused; an ocean run, frozen or migrating, writes the sea
level beside U and phi and restarts alike; the migrating run's growing cap
moves the shorelines (the ocean's share of the area changes from node to
node). `sl3d kernel`: its kernels block is checked and refused where a
kernel is not built; on the GPU each measurement's value is the solve's
field read there and the load kernels pair with the run's loads to it."""

import json
import pathlib
import subprocess

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def sl3d():
    import __graft_entry__

    __graft_entry__.build()
    from sl3dpp_gb300 import build

    return build.APP


def run(binary, mode, config, tmp_path, name="config.json", timeout=600):
    path = tmp_path / name
    path.write_text(json.dumps(config))
    return subprocess.run([str(binary), mode, str(path)], capture_output=True, text=True, timeout=timeout)


def base(tmp_path, lmax=8, nodes=5, **extra):
    config = {
        "model": {"earth": "standard", "elements": 20},
        "mesh": {"lmax": lmax, "ngll": 5},
        "lateral": {"viscosity": {"seed": 3, "degree": 4, "rms": 0.8}},
        "forcing": {"ice": {"cap_degrees": 15, "thickness_m": 2000, "ramp_nodes": 4}},
        "time": {"step_yr": 500, "nodes": nodes},
        "solve": {"scheme": "sdirk2", "precision": "fp64", "rtol": 1e-10, "max_iterations": 60},
        "output": {"file": str(tmp_path / "surface.txt")},
    }
    config.update(extra)
    return config


def run_hash(result):
    assert result.returncode == 0, result.stderr
    return result.stdout.split("run hash ")[1].split(",")[0]


def test_check_reads_the_config_and_hashes_what_decides_the_run(sl3d, tmp_path):
    cfg = base(tmp_path)
    h = run_hash(run(sl3d, "check", cfg, tmp_path))
    # key order and the steering members leave the hash alone
    steered = dict(reversed(list(base(tmp_path).items())))
    steered.update(checkpoint={"directory": str(tmp_path / "ck"), "stride": 2}, restart=True, stop_after_node=2,
                   output={"file": str(tmp_path / "other.txt")})
    assert run_hash(run(sl3d, "check", steered, tmp_path)) == h
    # a deciding member changes it
    other = base(tmp_path)
    other["lateral"]["viscosity"]["rms"] = 0.9
    assert run_hash(run(sl3d, "check", other, tmp_path)) != h
    other = base(tmp_path, nodes=6)
    assert run_hash(run(sl3d, "check", other, tmp_path)) != h


@pytest.mark.parametrize("change,text", [
    (lambda c: c.update(colour="blue"), "unknown member \"colour\""),
    (lambda c: c["solve"].update(scheme="leapfrog"), "solve.scheme"),
    (lambda c: c.pop("model"), "a model is required"),
    (lambda c: c["time"].update(step_yr=-1), "step_yr > 0"),
    (lambda c: c.update(restart=True), "checkpoint directory"),
    (lambda c: c["ocean"].update(rotation="sideways") if "ocean" in c else c.update(ocean={"rotation": "sideways"}),
     "ocean.rotation"),
    (lambda c: c.update(ocean={"shorelines": "wandering"}), "ocean.shorelines"),
    (lambda c: c.update(ocean={"shorelines": "migrating", "depth_m": -5}), "ocean.depth_m"),
])
def test_check_refuses_bad_configs(sl3d, tmp_path, change, text):
    cfg = base(tmp_path)
    change(cfg)
    result = run(sl3d, "check", cfg, tmp_path)
    assert result.returncode == 2 and text in result.stderr, result.stderr


def test_check_refuses_broken_json(sl3d, tmp_path):
    path = tmp_path / "broken.json"
    path.write_text('{"model": {"earth": "standard"},}')
    result = subprocess.run([str(sl3d), "check", str(path)], capture_output=True, text=True)
    assert result.returncode == 2 and "offset" in result.stderr


def table(path):
    return np.loadtxt(path, comments="#")


@pytest.mark.gpu
def test_gpu_solve_is_the_library_evolution(gpu, sl3d, tmp_path):
    import torch

    from sl3dpp_gb300 import configs
    from sl3dpp_gb300.grid import SurfaceGrid
    from sl3dpp_gb300.viscoelastic3d import Evolution3D, Options, Viscoelastic3D, standard_earth

    lmax, nodes = 8, 5
    coeffs = configs.delta_coefficients(lmax, 4, 0.8, 7)
    (tmp_path / "delta.bin").write_bytes(np.ascontiguousarray(coeffs, dtype=np.complex128).tobytes())
    cfg = base(tmp_path, lmax, nodes)
    cfg["lateral"] = {"viscosity": {"coefficients": str(tmp_path / "delta.bin")}}
    result = run(sl3d, "solve", cfg, tmp_path)
    assert result.returncode == 0, result.stdout + result.stderr
    got = table(tmp_path / "surface.txt")
    # the same run through the library's Python binding
    op = Viscoelastic3D(standard_earth(20), Options.defaults(lmax, 5, rtol=1e-10, max_iterations=60))
    pattern = SurfaceGrid(lmax, 0, 1.5).SynthesiseBatch(torch.tensor(coeffs, device=gpu), 1)
    ind = torch.tensor(configs.delta_indicator(op.radius), device=gpu)
    op.set_delta((ind[:, None] * pattern[None, :]).contiguous().view(-1))
    exact = SurfaceGrid(lmax, 0, 1.0)
    cap = configs.cap_field(exact.theta, exact.nphi, 15.0, 2000.0)
    full = (exact.ExpandBatch(torch.tensor(cap, device=gpu), 1) / op.surface_density_scale).cpu().numpy()
    times = np.arange(nodes) * 500 * configs.SECONDS_PER_YEAR / op.time_scale
    loads = np.minimum(np.arange(nodes), 4)[:, None] / 4 * full[None, :]
    want = Evolution3D(op, "sdirk2").Run(times, loads)
    lm = (lmax + 1) * (lmax + 2) // 2
    U = (got[:, 4] + 1j * got[:, 5]).reshape(nodes, lm) / op.length_scale
    phi = (got[:, 6] + 1j * got[:, 7]).reshape(nodes, lm) / (op.length_scale / op.time_scale) ** 2
    assert np.max(np.abs(U - want["U"])) <= 1e-15 * np.max(np.abs(want["U"]))
    assert np.max(np.abs(phi - want["phi"])) <= 1e-15 * np.max(np.abs(want["phi"]))


@pytest.mark.gpu
@pytest.mark.parametrize("ocean", ["none", "frozen", "migrating"])
def test_gpu_restart_continues_the_run_bit_for_bit(gpu, sl3d, tmp_path, ocean):
    extra = {} if ocean == "none" else {"ocean": {"land_fraction": 0.3, "seed": 11, "rotation": "axial",
                                                  "shorelines": ocean}}
    whole = base(tmp_path, nodes=6, **extra)
    whole["output"] = {"file": str(tmp_path / "whole.txt")}
    whole["checkpoint"] = {"directory": str(tmp_path / "ck_whole"), "stride": 2}
    assert run(sl3d, "solve", whole, tmp_path).returncode == 0
    part = base(tmp_path, nodes=6, **extra)
    part["output"] = {"file": str(tmp_path / "resumed.txt")}
    part["checkpoint"] = {"directory": str(tmp_path / "ck"), "stride": 2}
    part["stop_after_node"] = 3
    first = run(sl3d, "solve", part, tmp_path)
    assert first.returncode == 0 and "stopped after node 3" in first.stdout, first.stdout + first.stderr
    assert not (tmp_path / "resumed.txt").exists()
    assert sorted(p.name for p in (tmp_path / "ck").glob("*.ckpt")) == ["node_000000.ckpt", "node_000002.ckpt"]
    part.pop("stop_after_node")
    part["restart"] = True
    second = run(sl3d, "solve", part, tmp_path)
    assert second.returncode == 0 and "resumed after node 2" in second.stdout, second.stdout + second.stderr
    assert (tmp_path / "resumed.txt").read_bytes() == (tmp_path / "whole.txt").read_bytes()
    columns = table(tmp_path / "whole.txt").shape[1]
    assert columns == (8 if ocean == "none" else 10)
    # another run's checkpoints are refused
    other = dict(part)
    other["lateral"] = {"viscosity": {"seed": 4, "degree": 4, "rms": 0.8}}
    refused = run(sl3d, "solve", other, tmp_path)
    assert refused.returncode == 1 and "belongs to another run" in refused.stderr, refused.stderr


@pytest.mark.gpu
def test_gpu_migrating_run_moves_the_shorelines(gpu, sl3d, tmp_path):
    """A cap growing to 500 m over a quarter of the sphere, 70% of which is
    ocean up to 1.5 km deep: the ice grounds where it outweighs the water
    column, deeper as it thickens, and the falling sea level dries the
    shallowest coasts, so the ocean's share of the area changes from node to
    node; node 0 is the undisturbed background (zero response)."""
    cfg = base(tmp_path, nodes=5, ocean={"land_fraction": 0.3, "seed": 11, "rotation": "axial",
                                         "shorelines": "migrating", "depth_m": 1500})
    # a cap over a quarter of the sphere, thickening through the shallower
    # depths (2 km would take about 900 m of sea level and dry this ocean)
    cfg["forcing"] = {"ice": {"cap_degrees": 60, "thickness_m": 500, "ramp_nodes": 4}}
    result = run(sl3d, "solve", cfg, tmp_path)
    assert result.returncode == 0, result.stdout + result.stderr
    fractions = [float(line.split("ocean fraction ")[1]) for line in result.stdout.splitlines()
                 if "ocean fraction" in line]
    assert len(fractions) == 4 and len(set(fractions)) > 1, fractions
    got = table(tmp_path / "surface.txt")
    assert np.all(got[got[:, 0] == 0][:, 4:] == 0.0)
    assert np.max(np.abs(got[got[:, 0] == 4][:, 8:10])) > 0.0


# -- sl3d kernel ---------------------------------------------------------------------------------------

def kernel_config(tmp_path, **kernels):
    cfg = base(tmp_path, nodes=5)
    block = {"method": "discrete", "parameters": ["load", "tide", "viscosity"], "output": str(tmp_path / "kernels"),
             "measurements": [{"type": "displacement_point", "name": "uplift", "latitude": 63.2, "longitude": -20.5},
                              {"type": "potential_cap", "name": "geoid", "latitude": 70.0, "longitude": 10.0,
                               "width_deg": 8.0, "time": 1500.0}]}
    block.update(kernels)
    cfg["kernels"] = block
    return cfg


def test_check_reads_a_kernel_config(sl3d, tmp_path):
    result = run(sl3d, "check", kernel_config(tmp_path), tmp_path)
    assert result.returncode == 0, result.stderr
    assert "kernels of 2 measurement(s)" in result.stdout
    # the kernels block steers the run, it does not decide it
    assert run_hash(result) == run_hash(run(sl3d, "check", base(tmp_path, nodes=5), tmp_path))


@pytest.mark.parametrize("change,text", [
    (lambda c: c.update(ocean={}), "under an ocean are not built"),
    (lambda c: c["kernels"].update(method="continuous"), "\"continuous\" is not built"),
    (lambda c: c["kernels"].update(parameters=["ice"]), "\"ice\" needs an ocean"),
    (lambda c: c["kernels"].update(parameters=["moduli"]), "\"moduli\" is not built"),
    (lambda c: c["kernels"].update(parameters=["load", "load"]), "named twice"),
    (lambda c: c["kernels"].update(parameters=[]), "at least one"),
    (lambda c: c["kernels"].pop("output"), "kernels.output"),
    (lambda c: c["kernels"]["measurements"][0].update(type="relative_sea_level_point"), "needs an ocean"),
    (lambda c: c["kernels"]["measurements"][0].update(time=250.0), "not a node"),
    (lambda c: c["kernels"]["measurements"][1].pop("width_deg"), "width_deg > 0"),
    (lambda c: c["kernels"]["measurements"][1].update(name="uplift"), "named twice"),
    (lambda c: c["kernels"]["measurements"][0].update(name="../up"), "measurement.name"),
])
def test_check_refuses_bad_kernel_configs(sl3d, tmp_path, change, text):
    cfg = kernel_config(tmp_path)
    change(cfg)
    result = run(sl3d, "check", cfg, tmp_path)
    assert result.returncode == 2 and text in result.stderr, result.stderr


@pytest.mark.gpu
def test_gpu_kernel_values_and_kernels_are_the_runs(gpu, sl3d, tmp_path):
    """`sl3d kernel`: each measurement's value is the solve's surface field
    read there (a point by the orthonormal harmonics, a Gaussian cap by its
    degree weights); the load kernels pair with the run's loads to that
    value (dJ = sum_n int K_n sigma_n dS); the viscosity kernel is the
    library adjoint's gradient over the samples' volumes, in SI."""
    import torch
    from scipy.special import sph_harm_y

    from sl3dpp_gb300 import configs
    from sl3dpp_gb300.grid import SurfaceGrid
    from sl3dpp_gb300.viscoelastic3d import Evolution3D, Options, Viscoelastic3D, standard_earth

    lmax, nodes = 8, 5
    cfg = kernel_config(tmp_path)
    solved = run(sl3d, "solve", cfg, tmp_path)
    assert solved.returncode == 0, solved.stdout + solved.stderr
    result = run(sl3d, "kernel", cfg, tmp_path)
    assert result.returncode == 0, result.stdout + result.stderr
    got = table(tmp_path / "surface.txt")
    lm = (lmax + 1) * (lmax + 2) // 2
    U = (got[:, 4] + 1j * got[:, 5]).reshape(nodes, lm)
    phi = (got[:, 6] + 1j * got[:, 7]).reshape(nodes, lm)
    ls = np.concatenate([[l] * (l + 1) for l in range(lmax + 1)])
    ms = np.concatenate([list(range(l + 1)) for l in range(lmax + 1)])
    w = np.where(ms == 0, 1.0, 2.0)

    def at(coeffs, lat, lon, b=None):
        Y = sph_harm_y(ls, ms, np.radians(90.0 - lat), np.radians(lon))
        b = np.ones(lmax + 1) if b is None else b
        return float(np.sum(w * b[ls] * (coeffs * Y).real))

    def value(name):
        for line in (tmp_path / "kernels" / f"{name}_summary.txt").read_text().splitlines():
            if line.startswith("value "):
                return float(line.split()[1])

    uplift = at(U[nodes - 1], 63.2, -20.5)
    assert abs(value("uplift") - uplift) < 1e-9 * abs(uplift)
    d = np.linspace(0.0, np.pi, 40001)
    wcap = np.radians(8.0)
    f = np.exp(-d ** 2 / (2 * wcap ** 2)) * np.sin(d)
    Pl = [np.ones_like(d), np.cos(d)]
    for l in range(2, lmax + 1):
        Pl.append(((2 * l - 1) * np.cos(d) * Pl[-1] - (l - 1) * Pl[-2]) / l)
    trapezoid = getattr(np, "trapezoid", None) or np.trapz
    b = np.array([trapezoid(f * P, d) for P in Pl]) / trapezoid(f, d)
    geoid = at(phi[3], 70.0, 10.0, b)
    assert abs(value("geoid") - geoid) < 1e-7 * abs(geoid)

    # the load kernels pair with the run's loads (SI) to the value
    op = Viscoelastic3D(standard_earth(20), Options.defaults(lmax, 5, rtol=1e-10, max_iterations=60))
    exact = SurfaceGrid(lmax, 0, 1.0)
    cap = configs.cap_field(exact.theta, exact.nphi, 15.0, 2000.0)
    sigma = exact.ExpandBatch(torch.tensor(cap, device=gpu), 1).cpu().numpy()
    radius = max(layer.r1 for layer in standard_earth(20))
    for name, v in (("uplift", uplift), ("geoid", geoid)):
        k = table(tmp_path / "kernels" / f"{name}_load_kernels.txt")
        K = (k[:, 4] + 1j * k[:, 5]).reshape(nodes, lm)
        paired = sum(min(n, 4) / 4 * radius ** 2 * float(np.sum(w * (np.conj(K[n]) * sigma).real))
                     for n in range(nodes))
        assert abs(paired - v) < 1e-8 * abs(v), (name, paired, v)
        density = np.fromfile(tmp_path / "kernels" / f"{name}_viscosity_kernels.bin")
        assert density.size == op.values and np.all(np.isfinite(density)) and np.max(np.abs(density)) > 0
    # the tide kernels: written per node, none at degree 1
    tide = table(tmp_path / "kernels" / "uplift_tide_kernels.txt")
    T = (tide[:, 4] + 1j * tide[:, 5]).reshape(nodes, lm)
    assert np.all(np.isfinite(T)) and np.max(np.abs(T)) > 0 and np.all(T[:, 1:3] == 0)
