"""History file (punc/src/diagnostics.cpp:70-140, diagnostics.h:119-168): the
preamble lines and the row layout of the reference's history.dat."""
from puncpp_gb300 import punc


class _Obj:
    def __init__(self, potential, current, charge):
        self.potential, self.current, self.charge = potential, current, charge


class _Pop:
    def statistics(self):
        return [1.5, 0.25, 0.125, 0.0625]


def test_history_preamble_and_rows(tmp_path):
    f = tmp_path / "history.dat"
    objs = [_Obj(-2.0, 0.1, 3.0), _Obj(1.0, -0.5, 0.0)]
    h = punc.History(str(f), objs, dim=3, stats=True)
    h.save(7, 0.35, 1000.0, 998.0, 12.5, -3.25, objs, _Pop())
    h.close()
    lines = f.read_text().split("\n")
    assert lines[0] == "#:xaxis\tt"
    assert lines[1] == ("#:name\tn\tt\tne\tni\tKE\tPE\tV[0]\tI[0]\tQ[0]\tV[1]\tI[1]\tQ[1]"
                        "\tmean_e\tstdev_e\tmean_i\tstdev_i")
    assert lines[2].startswith('#:long\ttimestep\ttime\t"number of electrons"\t"number of ions"\t"kinetic energy"\t'
                               '"potential energy"\tvoltage\tcurrent\tcharge\tvoltage')
    assert lines[3] == "#:units\t1\ts\tm**(-3)\tm**(-3)\tJ\tJ\tV\tA\tC\tV\tA\tC\tm/s\tm/s\tm/s\tm/s"
    cols = lines[4].split("\t")
    assert cols[0] == "7" and len(cols) == 1 + 5 + 6 + 4
    assert cols[1] == "3.4999999999999998e-01" and cols[6] == "-2.0000000000000000e+00"
    assert [float(c) for c in cols[1:]] == [0.35, 1000.0, 998.0, 12.5, -3.25, -2.0, 0.1, 3.0, 1.0, -0.5, 0.0,
                                            1.5, 0.25, 0.125, 0.0625]
    # continuing appends rows without a second preamble
    h = punc.History(str(f), objs, stats=False, continue_simulation=True)
    h.save(8, 0.4, 1.0, 2.0, 3.0, 4.0, objs)
    h.close()
    lines = f.read_text().split("\n")
    assert lines[5].startswith("8\t4.0000000000000002e-01") and lines[6] == ""


def test_state_file_round_trip(tmp_path):
    """State::save / load (punc/src/diagnostics.cpp:40-68): next step, time,
    charge and current of the object, default stream precision."""
    f = tmp_path / "state.dat"
    objs = [_Obj(0.0, 0.125, 3.5)]
    punc.State(f).save(41, 2.05, objs)
    assert f.read_text() == "42\t2.05\t3.5\t0.125\n"
    back = [_Obj(0.0, 0.0, 0.0)]
    n, t = punc.State(f).load(back)
    assert (n, t, back[0].charge, back[0].current) == (42, 2.05, 3.5, 0.125)
