"""The autotuner's table export / import (JSON, host only, no GPU): round trip, the candidate
check on import, and all-or-nothing loading."""
from __future__ import annotations

import json

import pytest

from multigpu_advectiondiffusion_gb300 import _native as N
from multigpu_advectiondiffusion_gb300 import solvers as S


def _entries():
    return sorted((e["kind"], e["variant"], e["nx"], e["ny"], e["nz"], e["a"], e["b"])
                  for e in json.loads(S.autotune_export())["entries"])


def _table(*entries, version=1):
    keys = ("kind", "variant", "nx", "ny", "nz", "a", "b")
    return json.dumps({"advdiff_autotune": version, "entries": [dict(zip(keys, e)) for e in entries]})


@pytest.fixture(autouse=True)
def clean_table():
    S.autotune_clear()
    yield
    S.autotune_clear()


def test_export_of_an_empty_table():
    assert json.loads(S.autotune_export()) == {"advdiff_autotune": 1, "entries": []}


def test_import_then_export_round_trip(tmp_path):
    rows = [(1, 5, 256, 256, 256, 4, 8), (2, 3, 128, 96, 64, 2, 16), (3, 1, 192, 192, 192, 16, 32),
            (4, 2, 64, 64, 64, 4, 4)]
    S.autotune_import(_table(*rows))
    assert _entries() == sorted(rows)
    p = tmp_path / "tune.json"
    S.autotune_save(p)
    S.autotune_clear()
    assert _entries() == []
    S.autotune_load(p)
    assert _entries() == sorted(rows)
    # a later import replaces the shape of the same problem
    S.autotune_import(_table((1, 5, 256, 256, 256, 2, 4)))
    assert (1, 5, 256, 256, 256, 2, 4) in _entries() and len(_entries()) == 4


@pytest.mark.parametrize("text", [
    _table((3, 1, 64, 64, 64, 32, 16)),          # heat-k block height outside {4, 8, 16}
    _table((2, 1, 64, 64, 64, 4, 3)),            # Burgers share outside {4, 8, 16, 32}
    _table((1, 1, 64, 64, 64, 0, 8)),            # no CTAs
    _table((9, 1, 64, 64, 64, 1, 8)),            # unknown kind
    _table((5, 23, 64, 64, 64, 3, 1)),           # steps per launch outside {1, 2}
    _table((5, 23, 64, 64, 64, 2, 8)),           # steps per launch with b != 1
    _table((1, 1, 0, 64, 64, 1, 8)),             # empty grid
    _table((1, 1, 64, 64, 64, 1, 8), version=2),
    '{"advdiff_autotune": 1, "entries": [{"kind": 1, "variant": 1, "nx": 8, "ny": 8, "nz": 8, "a": 1}]}',
    '{"advdiff_autotune": 1, "entries": [{"kind": 1, "variant": 1, "nx": 8, "ny": 8, "nz": 8, "a": 1, "b": 8, "c": 1}]}',
    '{"advdiff_autotune": 1, "entries": []} trailing',
    '{"entries": []}',
    '[]',
    '',
])
def test_import_rejects_other_text_and_loads_nothing(text):
    S.autotune_import(_table((1, 7, 32, 32, 32, 1, 8)))
    before = _entries()
    with pytest.raises(N.AdvError) as e:
        S.autotune_import(text)
    assert e.value.status == N.ADV_ERR_INVALID_ARG
    assert _entries() == before


def test_a_bad_entry_after_good_ones_loads_none_of_them():
    with pytest.raises(N.AdvError):
        S.autotune_import(_table((1, 7, 32, 32, 32, 1, 8), (2, 1, 64, 64, 64, 2, 8), (3, 1, 64, 64, 64, 5, 8)))
    assert _entries() == []


def test_export_buffer_size_contract(native):
    import ctypes as C
    S.autotune_import(_table((1, 5, 256, 256, 256, 4, 8)))
    n = C.c_size_t(0)
    assert native.adv_autotune_export(None, 0, C.byref(n)) == N.ADV_OK and n.value > 10
    small = C.create_string_buffer(n.value - 1)
    assert native.adv_autotune_export(small, n.value - 1, C.byref(n)) == N.ADV_ERR_INVALID_ARG
    assert native.adv_autotune_export(None, 0, None) == N.ADV_ERR_INVALID_ARG
    assert native.adv_autotune_import(None) == N.ADV_ERR_INVALID_ARG


def test_steps_per_launch_entries_round_trip():
    """Table kind 5 (forward-Euler steps per launch of adv_heat_run) takes 1 or 2."""
    S.autotune_clear()
    S.autotune_import(_table((5, 23, 256, 256, 256, 2, 1), (5, 23, 96, 96, 96, 1, 1)))
    assert sorted(_entries()) == sorted([(5, 23, 256, 256, 256, 2, 1), (5, 23, 96, 96, 96, 1, 1)])
    S.autotune_clear()
