"""SQLite checkpoints (the reference's sql.py layout): a run resumed from a
checkpoint continues bit for bit, including pending spike deliveries, kinetic
states, the calcium pump and the clock."""
import sqlite3

import numpy as np
import pytest

import neuwon_gb300 as nw
from neuwon_gb300.morphology import random_tree
from tests.helpers import calcium_case, network_case

pytestmark = pytest.mark.gpu


def _network():
    m, _, _, _ = network_case([300, 200, 250, 150], 1500, seed=8, precision="f32", oracle=False, delay_lo=1.0,
                              delay_hi=6.0, currents=[0.5, 0.45, 0.4, 0.5])
    return m


def test_network_resumes_bit_for_bit(tmp_path):
    path = str(tmp_path / "net.sqlite")
    a = _network()
    a.advance(150)
    a.save_sqlite(path)
    a.advance(150)
    b = _network()
    b.load_sqlite(path)
    assert b._ctx.clock() == (150, 300)
    b.advance(150)
    for name in ("Segment.voltage", "Synapse.events", "Synapse.last_event", "Synapse.nmda_open", "Neuron.spike_count"):
        assert np.array_equal(a.get_data(name), b.get_data(name)), name
    assert a.get_data("Synapse.events").sum() > 0
    con = sqlite3.connect(path)
    tables = {r[0] for r in con.execute("SELECT name FROM sqlite_master WHERE type='table'")}
    assert {"Segment", "Neuron", "hh", "Synapse", "SpikeRing", "Model_cls_attrs"} <= tables
    assert con.execute("SELECT COUNT(*) FROM Segment").fetchone()[0] == 900
    con.close()
    a.close(); b.close()


@pytest.mark.parametrize("path_name", ["batched", "wide"])
def test_calcium_and_kinetic_resume_bit_for_bit(tmp_path, path_name):
    path = str(tmp_path / "ca.sqlite")

    def make():
        m, _, _ = calcium_case([random_tree(400, seed=21)], [(0, 0, 0.6, 0.0, 1e6)], precision="f64",
                               path=path_name, oracle=False)
        return m
    a = make()
    a.advance(300)
    a.save_sqlite(path)
    a.advance(200)
    b = make()
    b.load_sqlite(path)
    b.advance(200)
    for name in ("Segment.voltage", "Species.ca", "CaPump.state", "hh.m", "Neuron.spike_count"):
        assert np.array_equal(a.get_data(name), b.get_data(name)), name
    a.close(); b.close()


def test_checkpoint_rejects_another_structure(tmp_path):
    path = str(tmp_path / "x.sqlite")
    a = _network()
    a.advance(10)
    a.save_sqlite(path)
    m = nw.RxD_Model(time_step=0.1, temperature=6.3, mechanisms=[nw.HH])
    m.add_tree(random_tree(50, seed=1))
    m.insert_everywhere("hh")
    with pytest.raises(ValueError):
        m.load_sqlite(path)
    a.close(); m.close()
