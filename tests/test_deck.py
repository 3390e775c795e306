"""The .inp reader (giraffe_gb300.deck) against the writer and, where the
reference tree is present, against the reference's own tutorial decks read
as text.  CPU only."""
import os

import numpy as np
import pytest

from giraffe_gb300 import configs
from giraffe_gb300.deck import DeckError, read_deck, read_deck_file
from giraffe_gb300.model import NodalLoad

REF_INPUTS = os.path.join(os.environ.get("GIRAFFE_REFERENCE", "/root/reference"), "inputs")


def same_structure(a, b):
    assert np.array_equal(np.asarray(a.nodes), np.asarray(b.nodes))
    assert a.materials == b.materials
    assert a.sections == b.sections
    assert a.shell_sections == b.shell_sections
    assert a.cs == b.cs
    assert np.array_equal(a.beams.array(), b.beams.array())
    assert np.array_equal(a.shells.array(), b.shells.array())
    if a.constraints is None or b.constraints is None:
        assert a.constraints is None and b.constraints is None or \
            not np.asarray(a.constraints if a.constraints is not None else b.constraints).any()
    else:
        assert np.array_equal(np.asarray(a.constraints), np.asarray(b.constraints))
    assert len(a.loads) == len(b.loads)
    for x, y in zip(a.loads, b.loads):
        assert type(x) is type(y)
        if isinstance(x, NodalLoad):
            assert list(x.nodes) == list(y.nodes) and x.cs == y.cs
        else:
            assert list(x.shells) == list(y.shells) and int(x.area_update) == int(y.area_update)
        assert np.array_equal(x.table.times, y.table.times)
        assert np.array_equal(np.asarray(x.table.values, dtype=float), np.asarray(y.table.values, dtype=float))
    assert len(a.displacements) == len(b.displacements)
    for x, y in zip(a.displacements, b.displacements):
        assert list(x.nodes) == list(y.nodes) and x.cs == y.cs and x.angular == y.angular
        assert np.array_equal(x.table.times, y.table.times)
        assert np.array_equal(np.asarray(x.table.values, dtype=float), np.asarray(y.table.values, dtype=float))
    assert a.solution == b.solution
    assert a.next_steps == b.next_steps
    assert {int(k): float(v) for k, v in a.pretension.items()} == {int(k): float(v) for k, v in b.pretension.items()}
    assert {k: float(v) for k, v in a.criteria.items()} == {k: float(v) for k, v in b.criteria.items()}


@pytest.mark.parametrize("make", [
    configs.tutorial01, configs.cantilever_rollup, lambda: configs.tutorial10(0.2, 0.002, 1),
    lambda: configs.pipe_chain(25, 0.4, 0.03, [1e5, -2e4, 3e4]),
    lambda: configs.riser_chain(15, 0.35, 0.025, 1.0, 6.0, steps=30), lambda: configs.rotating_base("EulerVector"),
    configs.pretensioned_chain, configs.chain_sequence, lambda: configs.plate_release(3),
    lambda: configs.plate_dynamics(3, steps=10, rayleigh_alpha=8.0, rayleigh_beta=2e-5, update_rayleigh=1),
    lambda: configs.square_plate(3, steps=10, area_update=0), lambda: configs.square_plate(4, steps=20),
])
def test_written_deck_reads_back_the_same(make):
    s = make()
    same_structure(read_deck(s.to_inp()), s)


def test_sets_by_sequence_comments_and_skipped_blocks():
    s = configs.pipe_chain(4, 0.4, 0.03, [1e5, 0.0, 0.0])
    text = s.to_inp()
    # a node set written as a sequence, comments, and output blocks
    first = text.splitlines()
    k = next(i for i, ln in enumerate(first) if ln.startswith("NodeSet\t1\t"))
    first[k] = "NodeSet\t1\tNodes\t1\tSequence\tInitial\t1\tIncrement\t1   // the clamped end"
    text = "// header comment\n" + "\n".join(first) + "\nMonitor\tSample\t1\nMonitorNodes\t1\t9\n" \
        "PostFiles\nMagFactor\t1\nWriteMesh\t1\nContacts\t0\n"
    same_structure(read_deck(text), s)


def test_unsupported_content_is_refused():
    base = configs.pipe_chain(4, 0.4, 0.03, [1e5, 0.0, 0.0]).to_inp()
    with pytest.raises(DeckError, match="Truss_1"):
        read_deck(base.replace("Beam_1\t2\t", "Truss_1\t2\t"))
    mixed = configs.pipe_riser(4, steps=4)  # element 2 a Beam_1 inside the PipeLoad's set
    mixed.beams[1] = (2, 3, 4, mixed.add_material(2.1e11, 0.3, 7850.0), mixed.add_tube(0.3, 0.26), 0)
    del mixed.pipe_of[1]
    with pytest.raises(DeckError, match="every element must be a Pipe_1"):
        read_deck(mixed.to_inp())
    with pytest.raises(DeckError, match="Contacts"):
        read_deck(base + "Contacts\t1\nNSSS\t1\n")
    with pytest.raises(DeckError, match="solution step"):
        read_deck(base, step=2)


def _ref_deck(name):
    path = os.path.join(REF_INPUTS, name, name + ".inp")
    if not os.path.exists(path):
        pytest.skip("reference decks not present")
    return path


def test_reference_tutorial01_reads_as_the_built_config():
    same_structure(read_deck_file(_ref_deck("tutorial01")), configs.tutorial01())


def test_reference_tutorial10_reads_as_the_built_config():
    same_structure(read_deck_file(_ref_deck("tutorial10")), configs.tutorial10())


def test_reference_tutorial05_steps():
    """A Shell_1 strip with a tip load: a Static step, then a Dynamic step
    that starts from the first one's end state; the first step can be read
    alone, a later one cannot."""
    path = _ref_deck("tutorial05")
    s = read_deck_file(path)
    assert len(s.shells) == 400 and len(s.beams) == 0 and s.n_nodes == 861
    assert s.solution.type == 0 and s.solution.end_time == 1.0
    assert len(s.next_steps) == 1 and s.next_steps[0].type == 1 and s.next_steps[0].end_time == 1.4
    assert s.next_steps[0].beta == 0.3 and s.next_steps[0].time_step == 0.005
    assert int(np.asarray(s.constraints).sum()) == 21 * 6
    assert read_deck_file(path, step=1).next_steps == []
    with pytest.raises(DeckError, match="first solution step"):
        read_deck_file(path, step=2)
    same_structure(read_deck(s.to_inp()), s)


def test_zero_ic_and_step_dependent_tables():
    s = configs.chain_sequence()
    text = s.to_inp()
    assert "ZeroIC" in text
    r = read_deck(text)
    assert [x.zero_ic for x in r.next_steps] == [0, 1, 0]
    # a constraint released in the second step is refused
    k = text.index("NodalConstraint")
    bad = text[:k] + text[k:].replace("BoolTable\t1", "BoolTable\t1\t0", 1)
    with pytest.raises(DeckError, match="change between solution steps"):
        read_deck(bad)


def test_pipe_deck_round_trip():
    """Pipe_1 elements, PipeSections and PipeLoad written by to_inp read back
    into the same structure."""
    s = configs.pipe_riser(6, steps=8)
    r = read_deck(s.to_inp())
    assert r.pipe_of == s.pipe_of and r.pipe_sections == s.pipe_sections
    assert r.beams.array().tolist() == s.beams.array().tolist()
    assert len(r.loads) == 1 and r.loads[0].pipes == s.loads[0].pipes
    assert np.array_equal(r.loads[0].table.values, s.loads[0].table.values)
    assert r.to_inp() == s.to_inp()


def test_reference_tutorial04_reads():
    s = read_deck_file(_ref_deck("tutorial04"))
    assert len(s.beams) == 50 and len(s.pipe_of) == 50 and len(s.pipe_sections) == 1
    assert s.pipe_sections[0][-2:] == (0.65, 0.62)
    assert len(s.loads) == 2 and s.loads[1].pipes == list(range(50))
    assert [so.end_time for so in [s.solution] + s.next_steps] == [1.0, 2.0]


def test_reference_tutorial02_modal_step_reads():
    """tutorial02: 3,036 Shell_1 and a Modal step (12 modes)."""
    s = read_deck_file(_ref_deck("tutorial02"))
    assert s.modal is not None and s.modal.number_modes == 12 and s.modal.compute_eigenvectors == 1
    assert len(s.shells) == 3036 and s.n_free == 31323
    r = read_deck(s.to_inp())
    assert r.modal == s.modal


def test_monitor_file_text_round_trips():
    """The monitor writer's text: Node::WriteMonitor's header and %.6e
    columns, which read back as the values to that precision."""
    from giraffe_gb300.monitor import HEADER, node_lines
    rng = np.random.default_rng(3)
    lines = rng.normal(size=(5, 31)) * 10.0 ** rng.integers(-8, 6, size=(5, 31))
    text = node_lines(lines)
    rows = text.strip().split("\n")
    assert rows[0] == HEADER and len(rows[0].split("\t")) == 31
    back = np.array([[float(v) for v in r.split("\t")] for r in rows[1:]])
    assert np.allclose(back, lines, rtol=6e-7, atol=0)
