"""LAMMPS dumps and fix files in the reference's text formats, on hand-set
particle states: plotParticles_2D/3D (Output.jl:146-290; header, column order,
the two-space columns, elastic materials' zero plastic columns), EnergiesFix
(Fix.jl:248-270) and DisplacementFix (Fix.jl:37-102, 214-218), with Julia's
Float64 printing."""
import numpy as np

import jump_gb300 as J
from jump_gb300.output import OvitoOutput, plotParticles_2D, plotParticles_3D


def test_dump_2d(tmp_path):
    s1 = J.Solid2D(np.array([[0.25, 0.5], [0.75, 0.125]]), J.ElasticMaterial(1e3, 0.3, 1000.0, 2))
    s2 = J.Solid2D(np.array([[0.5, 0.5]]), J.ElastoPlasticMaterial(1e3, 0.3, 1000.0, 1.0, 0.0, 1))
    s1.stress[0] = [[1.5, 0.25], [0.25, -2.0]]
    s1.velocity[1] = [1e-5, 3.0]
    s2.mat.alpha[0] = 0.125
    s2.mat.vmStr[0] = 2.5
    s2.stress[0] = [[0.5, 0.0], [0.0, 0.25]]
    s2.damage[0] = 0.5
    outs = ["pstrain", "vonMises", "sigmaxx", "sigmayy", "pressure", "vx", "vy", "damage"]
    plotParticles_2D(OvitoOutput(10, str(tmp_path) + "/", outs), [s1, s2], [1.0, 2.0], [10, 20], 30)
    assert open(tmp_path / "dump_p.30.LAMMPS").read() == (
        "ITEM: TIMESTEP \n0\nITEM: NUMBER OF ATOMS\n3 \nITEM: BOX BOUNDS sm sm sm\n0 1.0\n0 2.0\n0 0\n"
        "ITEM: ATOMS id type x y z pstrain vonMises sigmaxx sigmayy pressure vx vy damage \n"
        "1 1 0.25 0.5 0 0 0 1.5 -2.0 -0.5 0.0  0.0  0.0  \n"
        "2 1 0.75 0.125 0 0 0 0.0 0.0 0.0 1.0e-5  3.0  0.0  \n"
        "3 2 0.5 0.5 0 0.125 2.5 0.5 0.25 0.75 0.0  0.0  0.5  \n")


def test_dump_3d(tmp_path):
    s = J.Solid3D(np.array([[0.25, 0.5, 0.75]]), J.ElastoPlasticMaterial(1e3, 0.3, 1000.0, 1.0, 0.0, 1))
    s.mat.alpha[0] = 0.25
    s.velocity[0] = [1.0, -2.0, 0.5]
    s.stress[0] = np.diag([1.0, 2.0, 4.0])
    out = OvitoOutput(5, str(tmp_path) + "/", ["pstrain", "vonMises", "vx", "vy", "vz", "pressure"])
    plotParticles_3D(out, [s], [1.0, 2.0, 3.0], [4, 8, 12], 0)
    assert open(tmp_path / "dump_p.0.LAMMPS").read() == (
        "ITEM: TIMESTEP \n0\nITEM: NUMBER OF ATOMS\n1 \nITEM: BOX BOUNDS sm sm sm\n0 1.0\n0 2.0\n0 3.0\n"
        "ITEM: ATOMS id type x y z pstrain vonMises vx vy vz pressure \n"
        "1 1 0.25 0.5 0.75 0.25 0.0 1.0  -2.0  0.5  7.0  \n")


def test_fix_files(tmp_path):
    s1 = J.Solid2D(np.array([[0.25, 0.5], [0.75, 0.125]]), J.ElasticMaterial(1e3, 0.3, 1000.0, 2))
    s2 = J.Solid2D(np.array([[0.5, 0.5], [0.75, 0.125]]), J.ElasticMaterial(1e3, 0.3, 1000.0, 2))
    e = J.EnergiesFix([s1], str(tmp_path / "energies.txt"))
    e.record(1e-5, 0.5, 2.0)
    e.close()
    assert open(tmp_path / "energies.txt").read() == "1.0e-5 0.5 2.0\n"
    d = J.DisplacementFix([s1, s2], [0.75, 0.125], str(tmp_path) + "/")
    assert d.index == (1, 1)  # a later solid with a matching particle replaces an earlier one
    s2.pos[1] += [0.25, -0.125]
    d.compute(0.5)
    d.close()
    assert open(tmp_path / "recorded-position.txt").read() == "0.5 0.25 -0.125\n"


def test_energies_fix_sums_in_the_reference_order(tmp_path):
    """KE += 0.5 m dot(v, v), SE += 0.5 V sum(stress .* strain), particle by particle
    (Fix.jl:248-270): the host EnergiesFix reproduces that loop bit for bit."""
    rng = np.random.default_rng(3)
    sols = []
    for n in (7, 0, 5):
        s = J.Solid2D(rng.random((n, 2)), J.ElasticMaterial(1e3, 0.3, 1000.0, max(n, 1)))
        s.mass[:] = rng.random(n)
        s.volume[:] = rng.random(n)
        s.velocity[:] = rng.standard_normal((n, 2))
        s.stress[:] = rng.standard_normal((n, 2, 2))
        s.strain[:] = rng.standard_normal((n, 2, 2))
        sols.append(s)
    KE = SE = 0.0
    for s in sols:
        for p in range(s.parCount):
            v = s.velocity[p]
            KE += 0.5 * s.mass[p] * (v[0] * v[0] + v[1] * v[1])
            st, ep = s.stress[p], s.strain[p]
            SE += 0.5 * s.volume[p] * (((st[0, 0] * ep[0, 0] + st[1, 0] * ep[1, 0]) + st[0, 1] * ep[0, 1])
                                       + st[1, 1] * ep[1, 1])
    e = J.EnergiesFix(sols, str(tmp_path / "e.txt"))
    e.compute(0.25)
    e.close()
    assert e.kinEnergy == [KE] and e.strEnergy == [SE]


def test_paths_are_concatenated_as_in_the_reference(tmp_path):
    """string(dir, name) (Output.jl:48,155; Fix.jl:61): no separator is added,
    an existing dir loses only dir * "*.LAMMPS", a missing one is made."""
    d = tmp_path / "out"
    d.mkdir()
    (d / "dump_p.7.LAMMPS").write_text("old")
    (d / "keep.txt").write_text("kept")
    OvitoOutput(1, str(d) + "/", ["vx"])
    assert sorted(p.name for p in d.iterdir()) == ["keep.txt"]
    s = J.Solid2D(np.array([[0.25, 0.5]]), J.ElasticMaterial(1e3, 0.3, 1000.0, 1))
    plotParticles_2D(OvitoOutput(1, str(tmp_path / "new") + "/", ["vx"]), [s], [1.0, 1.0], [2, 2], 3)
    assert (tmp_path / "new" / "dump_p.3.LAMMPS").is_file()
    J.DisplacementFix([s], [0.25, 0.5], str(tmp_path / "run_")).close()
    assert (tmp_path / "run_recorded-position.txt").is_file()
