"""yaml_io writes what it reads back: a property test over nested mappings, sequences and
scalars (text with control characters, quotes, non-ASCII; ints; floats incl. inf; bools; None),
and regression cases for the quoting rules."""
import importlib

import pytest

yio = importlib.import_module("3d_ravesim_gb300.yaml_io")


def test_round_trip_property():
    hyp = pytest.importorskip("hypothesis")
    st = pytest.importorskip("hypothesis.strategies")
    scal = st.one_of(st.none(), st.booleans(), st.integers(-10**12, 10**12), st.floats(allow_nan=False),
                     st.text(max_size=12))
    keys = st.one_of(st.text(min_size=1, max_size=8), st.integers(0, 1000))
    tree = st.recursive(scal, lambda ch: st.one_of(st.lists(ch, max_size=4), st.dictionaries(keys, ch, max_size=4)),
                        max_leaves=12)

    @hyp.settings(max_examples=400, deadline=None, suppress_health_check=list(hyp.HealthCheck))
    @hyp.given(st.dictionaries(keys, tree, min_size=1, max_size=5))
    def check(obj):
        assert yio.loads(yio.dumps(obj)) == obj

    check()


@pytest.mark.parametrize("value", ["a\x1eb", "line1\nline2", "tab\there", "é and ü", "say \"hi\"", "it's",
                                   "# not a comment", "a: b", "- dash", "\u2028", "back\\slash", "", " pad ",
                                   "null", "1e5", "true", "\x00", "\U0001f600"])
def test_strings_survive(value):
    doc = {"k": value, value or "e": [value, {"n": value}]}
    assert yio.loads(yio.dumps(doc)) == doc


def test_reads_comments_after_quoted_values():
    text = 'a: "x \\" # still x" # comment\nb: \'it\'\'s # in\' # out\nc: plain # gone\nd: it\'s\n'
    assert yio.loads(text) == {"a": 'x " # still x', "b": "it's # in", "c": "plain", "d": "it's"}


def test_rejects_bad_escapes():
    with pytest.raises(ValueError):
        yio.loads('a: "\\q"\n')
    with pytest.raises(ValueError):
        yio.loads('a: "\\x4"\n')
