"""Seeded random documents through the YAML subset of ``config.parse_yaml``:
nested block mappings with random indentation per level, blank and
comment-only lines, trailing comments, and every scalar kind the case
configurations use (integers, floats in plain and exponent form,
booleans, nulls, plain paths and titles, quoted strings that hold ':' and
'#').  The document is emitted from a known tree and must parse back to
it."""
import math

import numpy as np
import pytest

from tailor_gb300 import config

WORDS = ["case", "data", "sample", "FD-q", "run_1", "Tailor", "BiGlobal", "wavy", "wall"]


def _key(rng, used):
    while True:
        k = "".join(rng.choice(list("abcdefghijklmnopqrstuvwxyz_"), size=int(rng.integers(1, 10))))
        k = ("k" + k) if k[0] == "_" else k
        if k not in used and k not in ("true", "false", "null"):
            used.add(k)
            return k


def _value(rng):
    """(text, parsed value)"""
    kind = int(rng.integers(10))
    if kind == 0:
        v = int(rng.integers(-10 ** 9, 10 ** 9))
        return str(v), v
    if kind == 1:
        v = float(rng.standard_normal() * 10.0 ** rng.integers(-20, 20))
        return repr(v), v
    if kind == 2:
        m, e = int(rng.integers(1, 10)), int(rng.integers(-12, 12))
        return f"{m}e{e}", float(f"{m}e{e}")
    if kind == 3:
        v = bool(rng.integers(2))
        return ("true" if v else "false") if rng.random() < 0.5 else ("True" if v else "False"), v
    if kind == 4:
        return ("null", "~")[int(rng.integers(2))], None
    if kind == 5:  # a plain path or title
        parts = [str(rng.choice(WORDS)) for _ in range(int(rng.integers(1, 4)))]
        sep = "/" if rng.random() < 0.5 else " "
        s = sep.join(parts)
        return s, s
    if kind == 6:  # double-quoted, with ':' and '#'
        s = f"{rng.choice(WORDS)}: #{int(rng.integers(100))} {rng.choice(WORDS)}"
        return '"' + s + '"', s
    if kind == 7:  # single-quoted with an escaped quote
        s = f"{rng.choice(WORDS)}'s #{int(rng.integers(100))}"
        return "'" + s.replace("'", "''") + "'", s
    if kind == 8:  # a plain scalar with an apostrophe: text, not a quote
        s = f"{rng.choice(WORDS)}'s {rng.choice(WORDS)}"
        return s, s
    v = float(rng.integers(-1000, 1000))
    return repr(v), v


def _emit(rng, tree_depth, indent, lines):
    out, used = {}, set()
    step = int(rng.integers(2, 5))
    for _ in range(int(rng.integers(1, 7))):
        k = _key(rng, used)
        if rng.random() < 0.3:
            lines.append("")
        if rng.random() < 0.2:
            lines.append(" " * int(rng.integers(0, 6)) + "# a comment: with colon")
        comment = "  # trailing" if rng.random() < 0.3 else ""
        if tree_depth < 3 and rng.random() < 0.3:
            lines.append(" " * indent + f"{k}:{comment}")
            out[k] = _emit(rng, tree_depth + 1, indent + step, lines)
        else:
            text, v = _value(rng)
            lines.append(" " * indent + f"{k}: {text}{comment}")
            out[k] = v
    return out


def _equal(a, b):
    if isinstance(a, dict):
        return isinstance(b, dict) and a.keys() == b.keys() and all(_equal(a[k], b[k]) for k in a)
    if isinstance(a, float):
        return isinstance(b, float) and (a == b or (math.isnan(a) and math.isnan(b)))
    return type(a) is type(b) and a == b


@pytest.mark.parametrize("seed", range(40))
def test_random_documents_parse_back(seed):
    rng = np.random.default_rng(seed)
    lines = ["---"] if rng.random() < 0.3 else []
    tree = _emit(rng, 0, 0, lines)
    text = "\n".join(lines) + "\n"
    got = config.parse_yaml(text)
    assert _equal(tree, got), text


def test_quotes_and_comments():
    doc = ("title: Tailor's wavy wall  # the reference's sample\n"
           "a: 'it''s # kept'  # dropped\n"
           "b: \"x \\\" # kept\"  # dropped\n"
           "c: x#y\n")
    assert config.parse_yaml(doc) == {"title": "Tailor's wavy wall", "a": "it's # kept",
                                      "b": 'x " # kept', "c": "x#y"}


@pytest.mark.parametrize("doc,msg", [
    ("a: 1\n  b: 2\n", "bad indentation"),
    ("a:\n  b: 1\n   c: 2\n", "bad indentation"),
    ("a: 1\na: 2\n", "duplicate key"),
    ("a: [1, 2]\n", "unsupported YAML construct"),
    ("a: \"open\n", "unterminated quoted scalar"),
    ("\ta: 1\n", "tabs are not allowed"),
    ("just text\n", "expected 'key: value'"),
])
def test_malformed_documents_name_the_line(doc, msg):
    with pytest.raises(config.ConfigError, match=msg):
        config.parse_yaml(doc)
