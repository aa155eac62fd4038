"""The reference-facing callers above the C-ABI: the header-only C++ facade with the _2DTissue
interface (src/simulation/2DTissue.h:35-60, records of src/simulation/Struct.h:9-29) and the CLI
with the reference's flags (src/main.cpp:20-101).

CPU: a program written the way the reference's main.cpp drives _2DTissue compiles and links against
the library with only `using _2DTissue = tds::Tissue2D;`. GPU: the CLI and that program run, print
the order-parameter series, write the reference's CSV layout (IO.h:40-69), and agree with the
Python path on the same seed."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

CLI = os.path.join(ROOT, "2dtissue_gb300", "_build", "tds_cli")
BUILD = os.path.join(ROOT, "2dtissue_gb300", "_build")

# main.cpp's call pattern (main.cpp:76-98), unchanged except for the include and the alias
MAIN = r"""
#include <iostream>
#include "2dtissue_gb300/csrc/tissue.hpp"
using _2DTissue = tds::Tissue2D;
using System = tds::System;
int main() {
    bool save_data = false, particle_innenleben = false, optimized_monotile_boundary = false, use_kafka = false;
    std::string mesh_path = "";
    int particle_count = 300, step_count = 4;
    double v0 = 0.1;
    _2DTissue _2dtissue(save_data, particle_innenleben, optimized_monotile_boundary, mesh_path, particle_count,
                        step_count, v0, use_kafka);
    _2dtissue.start();
    int nbr = 0;
    while (!_2dtissue.is_finished()) {
        System data = _2dtissue.update();
        for (const auto& p : data.particles) nbr += p.neighbor_count;
        std::cout << "step " << data.order_parameter << " " << data.particles.size() << "\n";
    }
    for (double v : _2dtissue.get_order_parameter()) std::cout << "phi " << v << "\n";
    std::cout << "neighbours " << nbr << "\n";
    return 0;
}
"""


def _build_main(tmp_path):
    src = tmp_path / "main.cpp"
    src.write_text(MAIN)
    exe = tmp_path / "main"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I" + ROOT, "-I" + os.path.join(ROOT, "include"), str(src),
                        "-o", str(exe), "-L" + BUILD, "-l2dtissue_gb300", "-Wl,-rpath," + BUILD],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_reference_main_compiles_against_the_facade(tg, tmp_path):
    tg.lib()  # builds the library when it is missing
    _build_main(tmp_path)


def test_cli_rejects_unknown_flags(tg):
    tg.lib()
    r = subprocess.run([CLI, "--no-such-flag"], capture_output=True, text=True)
    assert r.returncode != 0 and "usage" in r.stderr


@pytest.mark.gpu
def test_reference_main_runs(tg, tmp_path):
    exe = _build_main(tmp_path)
    r = subprocess.run([str(exe)], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.split("\n")
    steps = [l for l in lines if l.startswith("step ")]
    phi = [float(l.split()[1]) for l in lines if l.startswith("phi ")]
    assert len(steps) == 4 and all(l.split()[2] == "300" for l in steps)
    assert len(phi) == 4 and all(0 <= v <= 1 for v in phi)
    # update()'s System.order_parameter is the step's value of the series
    np.testing.assert_allclose([float(l.split()[1]) for l in steps], phi, rtol=1e-5)


@pytest.mark.gpu
def test_cli_matches_the_python_path(tg, tmp_path):
    n, steps, dt, seed = 400, 5, 0.01, 3
    r = subprocess.run([CLI, "--step-count", str(steps), "--particle-count", str(n), "--step-time", str(dt),
                        "--seed", str(seed), "--save-data"], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    out = r.stdout.strip().split("\n")
    assert out[-1].startswith("Time taken")
    phi_cli = np.array([float(x) for x in out[:-1]])
    # the CLI's model values: the reference ctor defaults (sigma 0.41667, r_adh 1, k 1, k_adh 0.75,
    # v0 0.1, mu 1) with step_size = --step-time, tau 1, alignment 0.5, no noise
    p = tg.Params(radius=0.4166666666666667, k_rep=1.0, k_adh=0.75, r_max=1.0, v0=0.1, mu=1.0, tau=1.0,
                  align=0.5, eta=0.0, dt=dt)
    sim = tg.Simulation(tg.Mesh.ellipsoid(4, (2.0, 1.0, 1.0)), p, n, seed=seed)
    sim.start()
    sim.step(steps)
    phi_py = sim.order_parameter()[0][:, 0]
    np.testing.assert_allclose(phi_cli, phi_py, rtol=1e-5)
    # --save-data: save_matrix_to_csv's layout, 15 significant digits, files per step in ./data
    st = sim.get_state()
    uv = np.loadtxt(tmp_path / "data" / ("r_data_%d.csv" % steps), delimiter=",")
    r3 = np.loadtxt(tmp_path / "data" / ("r_data_3D_%d.csv" % steps), delimiter=",")
    nb = np.loadtxt(tmp_path / "data" / ("particles_color_%d.csv" % steps), dtype=int)
    assert uv.shape == (n, 2) and r3.shape == (n, 3) and nb.shape == (n,)
    np.testing.assert_allclose(uv, st["uv"], rtol=1e-14, atol=1e-15)
    np.testing.assert_allclose(r3, st["r3d"], rtol=1e-14, atol=1e-15)
    np.testing.assert_array_equal(nb, st["nbr"])
    assert len(os.listdir(tmp_path / "data")) == 3 * steps
    # the files are opened in append mode (IO.h:44): a second run into the same directory adds its
    # rows after the first run's (the same seed gives the same rows)
    r2 = subprocess.run([CLI, "--step-count", str(steps), "--particle-count", str(n), "--step-time", str(dt),
                         "--seed", str(seed), "--save-data"], capture_output=True, text=True, cwd=tmp_path)
    assert r2.returncode == 0, r2.stderr
    uv2 = np.loadtxt(tmp_path / "data" / ("r_data_%d.csv" % steps), delimiter=",")
    assert uv2.shape == (2 * n, 2)
    np.testing.assert_array_equal(uv2[:n], uv)
    np.testing.assert_array_equal(uv2[n:], uv)
