"""Checkpoints of the device state in SQLite, in the layout of the reference's
``sqlite3_save`` / ``sqlite3_load`` (neuwon/database/sql.py:78-129): one table
per class (Segment, Neuron, each mechanism, Synapse, ...), one row per
instance with its ``_idx``, one column per attribute, plus a class-attribute
table for the model (clock and shape).  Indices are the model's creation
order, as the reference saves after ``Database.sort()``; every value is read
back from the GPU and written to it again on load, so a run resumed from a
checkpoint continues bit for bit.
"""
import sqlite3

import numpy as np


def _table(cur, name, columns, rows):
    cols = ", ".join(f"{c} {t}" for c, t in columns)
    cur.execute(f"CREATE TABLE {name} (_idx BIGINT NOT NULL, {cols}, PRIMARY KEY (_idx))")
    ph = ", ".join("?" for _ in range(len(columns) + 1))
    names = ", ".join(["_idx"] + [c for c, _ in columns])
    cur.executemany(f"INSERT INTO {name} ({names}) VALUES ({ph})",
                    [(i,) + tuple(r) for i, r in enumerate(zip(*rows))])


def _column(cur, table, name, dtype=np.float64):
    cur.execute(f"SELECT {name} FROM {table} ORDER BY _idx")
    return np.array([r[0] for r in cur.fetchall()], dtype=dtype)


def _state_of(model):
    """Every stepped quantity, in creation / registration order."""
    m = model
    m._sync()
    m._flush_probes()
    st = {"Segment": {"voltage": m.get_data("Segment.voltage"),
                      "integral_voltage": m.get_data("Segment.integral_voltage")},
          "Neuron": {"AP_detected": m._ctx.get_data("Neuron.AP_detected", len(m._neuron_root), np.uint8),
                     "AP_state": m._ctx.get_data("Neuron.AP_state", len(m._neuron_root), np.uint8),
                     "spike_count": m._ctx.get_data("Neuron.spike_count", len(m._neuron_root), np.int64)}}
    for name, cls in m.mechanisms.items():
        if m._instance_count(name) == 0:
            continue
        from .kinetic import Kinetic
        if issubclass(cls, Kinetic):
            s = m.get_data(f"{name}.state")
            st[name] = {f"s{k}": s[:, k] for k in range(s.shape[1])}
        else:
            st[name] = {a: m.get_data(f"{name}.{a}") for a in ("m", "h", "n")}
    if m._syn is not None:
        st["Synapse"] = {a: m.get_data(f"Synapse.{a}") for a in
                         ("ampa_open", "nmda_open", "nmda_desensitized", "events", "last_event", "pulse_end")}
    if m._calcium is not None:
        st["Segment"]["ca"] = m.get_data("Species.ca")
        st["Segment"]["ca_derivative"] = m.get_data("Species.ca_derivative")
        if m._calcium.pump:
            s = m.get_data("CaPump.state")
            st["CaPump"] = {"e1": s[:, 0], "e1ca": s[:, 1], "e2": s[:, 2]}
    return st


def save_sqlite(model, filename):
    """Write the model's present state to an SQLite file (overwritten)."""
    m = model
    st = _state_of(m)
    open(filename, "w").close()
    con = sqlite3.connect(filename)
    cur = con.cursor()
    for table, cols in st.items():
        columns = [(c, "BIGINT" if np.asarray(v).dtype.kind in "iu" else "REAL") for c, v in cols.items()]
        rows = [np.asarray(v).tolist() for v in cols.values()]
        _table(cur, table, columns, rows)
    if m._syn is not None:
        nn = m._ctx.get_option("spike_neurons")
        words = m._ctx.get_option("synapse_ring_words")
        ring = m._ctx.get_data("Synapse.spike_ring", nn * words, np.uint32).reshape(nn, -1)
        cur.execute("CREATE TABLE SpikeRing (_idx BIGINT NOT NULL, bits BLOB NOT NULL, PRIMARY KEY (_idx))")
        cur.executemany("INSERT INTO SpikeRing (_idx, bits) VALUES (?, ?)",
                        [(j, ring[j].astype("<u4").tobytes()) for j in range(nn)])
    steps, ticks = m._ctx.clock()
    cur.execute("CREATE TABLE Model_cls_attrs (time_step REAL, precision TEXT, steps BIGINT, input_ticks BIGINT, "
                "num_segments BIGINT, num_neurons BIGINT, num_synapses BIGINT)")
    cur.execute("INSERT INTO Model_cls_attrs VALUES (?, ?, ?, ?, ?, ?, ?)",
                (m.time_step, m.precision, steps, ticks, m._n, len(m._neuron_root),
                 0 if m._syn is None else len(m._syn["pre"])))
    con.commit()
    con.close()


def load_sqlite(model, filename):
    """Restore a state written by ``save_sqlite`` into a model of the same
    structure (segments, neurons, mechanisms, synapses, time step)."""
    m = model
    m._sync()
    con = sqlite3.connect(filename)
    cur = con.cursor()
    cur.execute("SELECT time_step, precision, steps, input_ticks, num_segments, num_neurons, num_synapses "
                "FROM Model_cls_attrs")
    dt, precision, steps, ticks, nseg, nneu, nsyn = cur.fetchone()
    if nseg != m._n or nneu != len(m._neuron_root) or abs(dt - m.time_step) > 0 or \
            nsyn != (0 if m._syn is None else len(m._syn["pre"])):
        con.close()
        raise ValueError("checkpoint does not match this model's structure")
    ctx = m._ctx
    order = m._order
    seg = {c: _column(cur, "Segment", c) for c in ("voltage", "integral_voltage")}
    ctx.set_data("Segment.voltage", np.ascontiguousarray(seg["voltage"][order]))
    ctx.set_data("Segment.integral_voltage", np.ascontiguousarray(seg["integral_voltage"][order]))
    nn = len(m._neuron_root)
    ctx.set_data("Neuron.AP_detected", _column(cur, "Neuron", "AP_detected", np.uint8))
    ctx.set_data("Neuron.AP_state", _column(cur, "Neuron", "AP_state", np.uint8))
    ctx.set_data("Neuron.spike_count", _column(cur, "Neuron", "spike_count", np.uint32))
    from .kinetic import Kinetic
    for name, cls in m.mechanisms.items():
        if m._instance_count(name) == 0:
            continue
        if issubclass(cls, Kinetic):
            S = len(cls.scheme_factory().states)
            s = np.stack([_column(cur, name, f"s{k}") for k in range(S)], axis=1)
            ctx.set_data(m.kinetic_state_name(name), np.ascontiguousarray(s.ravel()))
        else:
            for a in ("m", "h", "n"):
                ctx.set_data(f"hh.{a}", _column(cur, name, a))
    if m._syn is not None:
        for a in ("ampa_open", "nmda_open", "nmda_desensitized"):
            ctx.set_data(f"Synapse.{a}", _column(cur, "Synapse", a))
        for a in ("events", "last_event", "pulse_end"):
            ctx.set_data(f"Synapse.{a}", _column(cur, "Synapse", a, np.int64).astype(np.float64))
        cur.execute("SELECT bits FROM SpikeRing ORDER BY _idx")
        ring = np.concatenate([np.frombuffer(r[0], dtype="<u4") for r in cur.fetchall()]).astype(np.uint32)
        ctx.set_data("Synapse.spike_ring", ring)
    if m._calcium is not None:
        for a, attr in (("ca", "Species.ca"), ("ca_derivative", "Species.ca_derivative")):
            vals = np.ascontiguousarray(_column(cur, "Segment", a)[order])
            ctx.call("nw_calcium_data", attr.encode(), vals.ctypes.data_as(__import__("ctypes").c_void_p), 1,
                     len(vals), 1)
        if m._calcium.pump:
            s = np.stack([_column(cur, "CaPump", c)[order] for c in ("e1", "e1ca", "e2")], axis=0)
            s = np.ascontiguousarray(s.ravel())
            ctx.call("nw_calcium_data", b"CaPump.state", s.ctypes.data_as(__import__("ctypes").c_void_p), 1, len(s), 1)
    con.close()
    ctx.set_option("set_steps", steps)
    m.input_hook.ticks = ticks
    m.advance_hook.ticks = steps
    m._dirty_probes = True
