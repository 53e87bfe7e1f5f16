"""The C++ operator runner (xnb-exec): deck parsing, the reference's block
structure and step order, and the error behaviour (no GPU needed: --dry-run)."""
import os
import subprocess

import numpy as np
import pytest

from exanbody_gb300 import build

HERE = os.path.dirname(os.path.abspath(__file__))
DECK = os.path.join(HERE, "decks", "lj_ni_golden.msp")


def xnb_exec(*args, cwd=None):
    exe = build.build_host() if os.path.exists(build.LIB) else None
    if exe is None:
        build.build()
        exe = build.EXEC
    return subprocess.run([exe, *args], capture_output=True, text=True, timeout=300, cwd=cwd)


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
    # simulation_epilog, then final_dump = dump_data_particles (dump-data.msp:31-43)
    assert ops[ops.index("check_values"):] == ["check_values", "timestep_file", "message", "print_dump_file",
                                               "message", "write_dump"]
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
def test_ni_golden_deck_through_the_operator_runner(tmp_path):
    """The reference-style regression deck passes its check_values on the GPU
    (and leaves its final dump in the working directory)."""
    r = xnb_exec(DECK, cwd=tmp_path)
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


def _deck_body(end, epilog="nop"):
    """The Ni deck without its golden check, ending at `end`."""
    text = open(DECK).read().split("simulation_epilog:")[0]
    return text.replace("simulation_end_iteration: 100", "simulation_end_iteration: %d" % end) + \
        "simulation_epilog: %s\n" % epilog


@pytest.mark.gpu
def test_restart_from_final_dump_through_read_dump(tmp_path):
    """final_dump writes particles_%09d.dump; a deck whose input_data is
    read_dump continues from it. 30 + 30 steps agree with 60 steps in one run to
    rounding (the restart re-bins particles, so pair orders may differ)."""
    from exanbody_gb300 import dump

    a, c = tmp_path / "a", tmp_path / "c"
    a.mkdir()
    c.mkdir()
    (a / "a.msp").write_text(_deck_body(30))
    r = xnb_exec(str(a / "a.msp"), cwd=a)
    assert r.returncode == 0, r.stdout + r.stderr
    first = a / "particles_000000031.dump"
    info = dump.read_info(first)
    assert info["timestep"] == 31 and info["n_particles"] == 16384
    ni_input = ("input_data:\n  - particle_types\n  - particle_type_add_properties:\n      Ni: { mass: 58.693 Da }\n"
                "  - read_dump: { filename: %s }\n" % first)
    body = _deck_body(61)
    body = body.replace(body[body.index("input_data:"): body.index("replicate_domain:")], ni_input + "\n")
    (a / "b.msp").write_text(body)
    r = xnb_exec(str(a / "b.msp"), cwd=a)
    assert r.returncode == 0, r.stdout + r.stderr
    (c / "c.msp").write_text(_deck_body(60))
    r = xnb_exec(str(c / "c.msp"), cwd=c)
    assert r.returncode == 0, r.stdout + r.stderr
    restarted = dump.read(a / "particles_000000062.dump")
    straight = dump.read(c / "particles_000000061.dump")
    assert restarted["info"]["physical_time"] == pytest.approx(straight["info"]["physical_time"] + 2e-3, rel=1e-12)
    o1, o2 = np.argsort(restarted["id"]), np.argsort(straight["id"])
    assert np.array_equal(restarted["id"][o1], straight["id"][o2])
    L = np.array(straight["info"]["domain"]["extent"]) - np.array(straight["info"]["domain"]["origin"])
    dr = restarted["r"][o1] - straight["r"][o2]
    dr -= L * np.round(dr / L)
    assert np.max(np.abs(dr)) < 1e-9
    assert np.max(np.abs(restarted["v"][o1] - straight["v"][o2])) < 1e-9
