"""ACE type-1 tables (scone_gb300/ace.py): synthetic nuclides written and read back, several tables
in one file, and SCONE's own H-1 table (IntegrationTestFiles/1001JEF311.ace, the 1001.03c table cut
out by tests/golden/make_golden.py into tests/golden/scone_h1_1001_03c.ace) read as aceCard reads it
(NuclearData/DataDecks/ACE/aceCard_class.f90:1454-1530) and run through the oracle to the cross
sections of aceNeutronDatabase_iTest.f90:183-197.  No GPU is used."""
import json
import os

import numpy as np
import pytest

from scone_gb300 import abi, ace, problems

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "scone_golden.json")))
H1_TABLE = os.path.join(os.path.dirname(__file__), "golden", "scone_h1_1001_03c.ace")


def test_synthetic_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    path = str(tmp_path / "lib.ace")
    nucs = [problems.synthetic_nuclide(rng, n, A) for n, A in ((500, 1.0), (2000, 15.86), (1200, 55.9))]
    starts = []
    for k, n in enumerate(nucs):
        starts.append(ace.write_table(path, f"{1001 + 1000 * k}.99c", n["A"], n["kT"], n["e"], n["xs"][:, 0],
                                      n["xs"][:, 1], n["xs"][:, 3], ext_mode="a"))
    assert starts[0] == 1 and starts[1] > starts[0] and starts[2] > starts[1]
    for k, (n, s) in enumerate(zip(nucs, starts)):
        r = ace.nuclide(path, s)
        assert r["zaid"] == f"{1001 + 1000 * k}.99c"
        np.testing.assert_allclose(r["e"], n["e"], rtol=1e-10, atol=0)
        np.testing.assert_allclose(r["xs"], n["xs"], rtol=1e-10, atol=0)
        assert abs(r["A"] - n["A"]) < 1e-6 and abs(r["kT"] / n["kT"] - 1.0) < 1e-4
        t = ace.read_table(path, s)
        (cap,) = ace.reactions(t)
        assert cap["mt"] == 102 and cap["ty"] == 0 and cap["ie"] == 1
        np.testing.assert_allclose(cap["xs"], n["xs"][:, 3], rtol=1e-10)


def test_written_table_drives_the_oracle(tmp_path, oracle_mod):
    """A nuclide read back from its ACE table gives the oracle the cross sections it was written with."""
    rng = np.random.default_rng(4)
    n = problems.synthetic_nuclide(rng, 800, 1.0)
    path = str(tmp_path / "h.ace")
    ace.write_table(path, "1001.98c", n["A"], n["kT"], n["e"], n["xs"][:, 0], n["xs"][:, 1], n["xs"][:, 3])
    r = ace.nuclide(path)
    ce = problems.ce_data([dict(e=r["e"], xs=r["xs"], A=r["A"], kT=r["kT"])], [[(0, 1.0)]])
    gb = problems.GeometryBuilder()
    box = gb.surface(abi.BOX, 0.0, 0.0, 0.0, 1.0, 1.0, 1.0)
    gb.root_universe(box, 1, bc=[abi.BC_REFLECTIVE] * 6)
    o = oracle_mod.Oracle(problems.Problem(gb.arrays(), None, ce=ce))
    for k in (0, 10, 400, 799):
        np.testing.assert_allclose(o.ce_micro(0, n["e"][k]), n["xs"][k], rtol=1e-10)


def test_rejects_malformed_tables(tmp_path):
    with pytest.raises(ValueError):
        ace.write_table(str(tmp_path / "x.ace"), "1.00c", 1.0, 1e-8, [1.0, 0.5], [1, 1], [1, 1], [0, 0])


def test_reads_scone_h1_table(oracle_mod):
    r = ace.nuclide(H1_TABLE)
    assert r["zaid"] == "1001.03c"
    g = GOLD["h1_ace"]
    assert np.array_equal(r["e"], g["e"]) and np.array_equal(r["xs"][:, 0], g["total"])
    assert np.array_equal(r["xs"][:, 1], g["elastic"]) and np.array_equal(r["xs"][:, 3], g["absorption"])
    assert not r["xs"][:, 2].any()                              # H-1 has no inelastic reactions
    ce = problems.ce_data([dict(e=r["e"], xs=r["xs"], A=r["A"], kT=r["kT"])], [[(0, 1.0)]])
    gb = problems.GeometryBuilder()
    box = gb.surface(abi.BOX, 0.0, 0.0, 0.0, 1.0, 1.0, 1.0)
    gb.root_universe(box, 1, bc=[abi.BC_REFLECTIVE] * 6)
    o = oracle_mod.Oracle(problems.Problem(gb.arrays(), None, ce=ce))
    m = o.ce_micro(0, 5.6e-3)
    assert abs(1.0 - 19.731020820000000 / m[0]) < 1e-6 and abs(1.0 - 6.948036800000000e-04 / m[3]) < 1e-6
