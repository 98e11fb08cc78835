"""CPU tests of periodic boxes (<Translate_to>): known-answer jumps of the
restatement of geometry_2d::translate (include/geometry_2d.hpp:366-493), the
engine's host tables for a periodic geometry, and properties of the
restatement on the periodic bar (the layout of the reference's example_bar)."""
import numpy as np
import pytest

import btegpu
import pyoracle
import synth


@pytest.fixture(scope="module")
def bar():
    return synth.periodic_bar_geometry()  # strips 0-9, right 10, left 11, reservoirs 12, 13


def test_translate_wraps_right_to_left(bar):
    assert pyoracle.translate(bar, 10, 20.0, 13.0, 1.0, 0.5) == (3, (0.0, 13.0))


def test_translate_wraps_left_to_right(bar):
    assert pyoracle.translate(bar, 11, 0.0, 37.5, -2.0, 0.1) == (9, (20.0, 37.5))


@pytest.mark.parametrize("vy,box", [(0.5, 3), (-0.5, 2)])
def test_translate_at_a_strip_border_goes_ahead(bar, vy, box):
    """On the line between strips 2 and 3 both contacts meet the jump; the
    candidate that lies ahead of the velocity wins."""
    assert pyoracle.translate(bar, 10, 20.0, 12.0, 1.0, vy) == (box, (0.0, 12.0))


def test_translate_outside_a_periodic_box_is_an_error(bar):
    with pytest.raises(btegpu.BteError):
        pyoracle.translate(bar, 3, 10.0, 13.0, 1.0, 0.5)


def test_periodic_geometry_leaves_the_grid_path(built, bar):
    assert btegpu.debug_grid(bar)[0] == 0
    assert np.array_equal(btegpu.debug_geometry(bar), pyoracle.geometry_dump(bar))


def test_periodic_restatement_properties():
    case = synth.periodic_case(n_particles=1500)
    a = pyoracle.rta_run(case, nthreads=1)
    b = pyoracle.rta_run(case, nthreads=4)
    assert np.array_equal(a["exact"], b["exact"])
    assert a["translations"] > 0 and a["translations"] == b["translations"]
    assert a["wall_hits"] == 0          # the bar has no void border
    assert a["absorbed"] > 0
    # periodic boxes hold no particle time (a particle leaves them at once)
    assert np.all(a["gz"][10:12] == 0.0)


def test_periodic_profile_falls_from_hot_to_cold():
    case = synth.periodic_case(n_particles=6000, maxtime=300.0)
    r = pyoracle.rta_run(case, nthreads=8)
    T = r["temperature"][:10, -10:].mean(axis=1)
    slope = np.polyfit(np.arange(10), T, 1)[0]
    assert slope < 0 and T[0] > T[-1]


def test_geometry_xml_writes_translate_to(tmp_path, bar):
    p = tmp_path / "beam.xml"
    synth.write_geometry_xml(str(p), bar)
    text = p.read_text()
    assert text.count("<Translate_to") == 2
    assert '<Translate_to id="11">' in text and "-20.0 0.0 0.0" in text
