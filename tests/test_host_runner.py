"""The C++ operator runner (xnb-exec): deck parsing, the reference's block
structure and step order, and the error behaviour (no GPU needed: --dry-run)."""
import os
import subprocess

import pytest

from exanbody_gb300 import build

HERE = os.path.dirname(os.path.abspath(__file__))
DECK = os.path.join(HERE, "decks", "lj_ni_golden.msp")


def xnb_exec(*args):
    exe = build.build_host() if os.path.exists(build.LIB) else None
    if exe is None:
        build.build()
        exe = build.EXEC
    return subprocess.run([exe, *args], capture_output=True, text=True, timeout=120)


def test_dry_run_follows_the_numerical_scheme():
    r = xnb_exec("--dry-run", DECK)
    assert r.returncode == 0, r.stderr
    ops = [l for l in r.stdout.splitlines() if not l.startswith("xnb-exec") and l != "nop"]
    # input_data, nbh_dist, first_iteration
    head = ops[: ops.index("next_time_step") + 1]
    assert head[:4] == ["particle_types", "particle_type_add_properties", "domain", "init_rcb_grid"]
    assert "lattice" in head and "gaussian_noise_r" in head and "nbh_dist" in head
    assert head[head.index("init_particles"):] == [
        "init_particles", "print_grid", "zero_particle_force", "lennard_jones_force", "update_force_from_ghost",
        "divide_force_by_type_scalar", "simulation_stats", "print_simulation_stats", "next_time_step"]
    # one numerical_scheme step (numerical-scheme.msp:21-25 with update-particles.msp:75-78)
    step = ops[len(head): len(head) + 11]
    assert step == ["push_f_v_r", "push_f_v", "particle_displ_over", "ghost_update_r", "zero_particle_force",
                    "lennard_jones_force", "update_force_from_ghost", "divide_force_by_type_scalar", "push_f_v",
                    "next_time_step", "sim_continue"]
    assert ops.count("push_f_v_r") == 100
    assert ops[-1] == "check_values"
    assert "done, 100 steps" in r.stdout


def test_unknown_operator_is_an_error(tmp_path):
    deck = tmp_path / "bad.msp"
    deck.write_text("simulation: main\nmain:\n  - no_such_operator\n")
    r = xnb_exec("--dry-run", str(deck))
    assert r.returncode == 1 and "no_such_operator" in r.stderr


def test_units_and_overrides(tmp_path):
    deck = tmp_path / "u.msp"
    deck.write_text(
        "simulation: main\n"
        "global: { dt: 2 fs, rcut_max: 0.41 nm, rcut_inc: 2.0 ang }\n"
        "main:\n  - global\n  - nbh_dist\n  - my_block\n"
        "my_block:\n  - push_f_v: { dt_scale: 0.25 }\n"
        "+my_block:\n  - sim_continue\n")
    r = xnb_exec("--dry-run", str(deck))
    assert r.returncode == 0, r.stderr
    assert r.stdout.splitlines()[:3] == ["nbh_dist", "push_f_v", "sim_continue"]


@pytest.mark.gpu
def test_ni_golden_deck_through_the_operator_runner():
    """The reference-style regression deck passes its check_values on the GPU."""
    r = xnb_exec(DECK)
    assert r.returncode == 0, r.stdout + r.stderr
    vals = {}
    for line in r.stdout.splitlines():
        if line.startswith("** "):
            name = line.split()[1]
            vals[name] = float(line.split("=")[1].split("/")[0])
    assert vals["Position"] < 1e-9 and vals["Acceleration"] < 1e-6 and vals["Velocity"] < 1e-8


def test_chained_force_operators(tmp_path):
    """A force block in the reference's form: zero_particle_force, then
    lennard_jones_force and gravitational_force (config { G }, rcut, with units)."""
    deck = tmp_path / "g.msp"
    deck.write_text(
        "simulation: main\n"
        "main:\n  - compute_all_forces_energy\n"
        "compute_force:\n"
        "  - lennard_jones_force\n"
        "  - gravitational_force:\n"
        "      config: { G: 6.67e-11 }\n"
        "      rcut: 2.5 ang\n")
    r = xnb_exec("--dry-run", str(deck))
    assert r.returncode == 0, r.stderr
    assert r.stdout.splitlines()[:3] == ["zero_particle_force", "lennard_jones_force", "gravitational_force"]
    bad = tmp_path / "b.msp"
    bad.write_text("simulation: main\nmain:\n  - gravitational_force: { rcut: 2.5 }\n")
    r = xnb_exec("--dry-run", str(bad))
    assert r.returncode == 1 and "config { G }" in r.stderr
