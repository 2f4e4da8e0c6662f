"""Strategy settings without a GPU (the reference's strategy.rs:311-407 and testing.rs hooks):
TLG_GEOM_STRATEGY parsing (one name, per-family lists, case-insensitive families, invalid values),
the precedence of this thread's setting over the environment, scoped per-family overrides and
their restoration, and that settings are per thread."""

import os
import subprocess
import sys
import threading

import pytest

import gridcl_gb300 as tg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def in_env(value, code):
    """Runs `code` in a fresh interpreter with TLG_GEOM_STRATEGY=value; returns its stdout lines."""
    env = dict(os.environ, TLG_GEOM_STRATEGY=value)
    r = subprocess.run([sys.executable, "-c", "import gridcl_gb300 as tg\n" + code], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    return r.stdout.split()


FAMS = "EVector Points Jacobian Normals FacetNormals PullBack".split()
SHOW = "print(*[tg.get_strategy(f) for f in %r])" % FAMS


def test_one_name_for_every_family():
    assert in_env("loops", SHOW) == ["loops"] * 6
    assert in_env("policy", SHOW) == ["auto"] * 6
    assert in_env("cooperative", SHOW) == ["cooperative"] * 6


def test_per_family_list():
    got = in_env("jacobian=sumfact, Points = direct,FACETNORMALS=shared", SHOW)
    assert got == ["auto", "direct", "sumfact", "auto", "shared", "auto"]


@pytest.mark.parametrize("value", ["bogus", "Jacobian=sumfact,Jacobian=loops", "Jacobian", "Faces=loops",
                                   "Jacobian=fast"])
def test_invalid_values_fail_loudly(value):
    code = ("try:\n    tg.get_strategy('Jacobian')\n    print('accepted')\n"
            "except tg.GridError as e:\n    print('rejected', 'TLG_GEOM_STRATEGY' in str(e))")
    assert in_env(value, code) == ["rejected", "True"]


def test_setting_wins_over_the_environment():
    code = ("with tg.with_strategy('direct', family='Points'):\n    print(tg.get_strategy('Points'))\n"
            "print(tg.get_strategy('Points'))\n"
            "with tg.with_strategy('policy'):\n    print(tg.get_strategy('Jacobian'))\n")
    assert in_env("Points=loops,Jacobian=sumfact", code) == ["direct", "loops", "auto"]


def test_scopes_nest_per_family_and_restore():
    before = {f: tg.get_strategy(f) for f in FAMS}
    with tg.with_strategy("loops"):
        with tg.with_strategy("sumfact", family="Jacobian"):
            assert tg.get_strategy("Jacobian") == "sumfact"
            assert tg.get_strategy("Points") == "loops"
        assert tg.get_strategy("Jacobian") == "loops"
    assert {f: tg.get_strategy(f) for f in FAMS} == before


def test_settings_are_per_thread():
    seen = []
    with tg.with_strategy("cooperative"):
        t = threading.Thread(target=lambda: seen.append(tg.get_strategy("Jacobian")))
        t.start()
        t.join()
        assert tg.get_strategy("Jacobian") == "cooperative"
    assert seen == [tg.get_strategy("Jacobian")]


def test_unknown_names():
    with pytest.raises(tg.GridError):
        tg.set_strategy("fastest")
    with pytest.raises(tg.GridError):
        tg.get_strategy("Faces")
