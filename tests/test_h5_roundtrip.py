"""Seeded round trips through the built-in HDF5 writer and reader: random
group trees (up to 200 links in one group, so several symbol-table nodes),
datasets of every writable element type and rank (scalars and empty
arrays included), and attributes of every writable kind."""
import numpy as np
import pytest

from tailor_gb300 import h5

DTYPES = [np.float64, np.int8, np.int16, np.int32, np.int64, np.uint8, np.uint16, np.uint32,
          np.uint64]


def _array(rng):
    dt = DTYPES[rng.integers(len(DTYPES))]
    rank = int(rng.integers(0, 4))
    shape = tuple(int(rng.integers(0, 5)) if rng.random() < 0.1 else int(rng.integers(1, 7))
                  for _ in range(rank))
    if dt == np.float64:
        return rng.standard_normal(shape) * 10.0 ** rng.integers(-300, 300)
    info = np.iinfo(dt)
    return rng.integers(info.min, info.max, size=shape, dtype=dt, endpoint=True)


def _attr(rng):
    k = int(rng.integers(5))
    if k == 0:
        return "".join(chr(c) for c in rng.integers(32, 127, size=int(rng.integers(0, 40))))
    if k == 1:
        return int(rng.integers(-2 ** 62, 2 ** 62))
    if k == 2:
        return float(rng.standard_normal())
    return _array(rng)


def _build(rng, g, expect, path, depth):
    for _ in range(int(rng.integers(0, 4))):
        g.attrs[f"a{rng.integers(1 << 30)}"] = _attr(rng)
    expect[path or "/"] = ("group", dict(g.attrs))
    width = int(rng.integers(1, 200)) if depth == 0 else int(rng.integers(0, 12))
    for n in range(width):
        name = f"n{n}_{rng.integers(1 << 20)}"
        full = f"{path}/{name}"
        if depth < 2 and rng.random() < 0.2:
            _build(rng, g.group(name), expect, full, depth + 1)
        else:
            a = _array(rng)
            attrs = {f"d{i}": _attr(rng) for i in range(int(rng.integers(0, 3)))}
            g.dataset(name, a, attrs)
            expect[full] = (a, attrs)


def _same(x, y):
    if isinstance(x, str):
        return isinstance(y, str) and x == y
    x, y = np.asarray(x), np.asarray(y)
    return x.shape == y.shape and x.dtype == y.dtype and np.array_equal(x, y)


@pytest.mark.parametrize("seed", range(12))
def test_random_tree_round_trip(tmp_path, seed):
    rng = np.random.default_rng(seed)
    w = h5.Writer()
    expect = {}
    _build(rng, w, expect, "", 0)
    path = tmp_path / "t.h5"
    w.write(path)
    with h5.File(path) as f:
        for name, (value, attrs) in expect.items():
            node = f if name == "/" else f[name]
            if isinstance(value, str) and value == "group":
                assert isinstance(node, h5.Group)
                got = node.attrs
            else:
                assert isinstance(node, h5.Dataset)
                assert _same(value, node[...]), name
                got = node.attrs
            assert set(got) == set(attrs), name
            for k, v in attrs.items():
                if isinstance(v, int):
                    assert int(got[k]) == v
                elif isinstance(v, float):
                    assert float(got[k]) == v
                else:
                    assert _same(v, got[k]), (name, k)
        # every written child is listed, and nothing else
        for name, (value, _) in expect.items():
            if isinstance(value, str) and value == "group":
                node = f if name == "/" else f[name]
                kids = {k for k in expect if k.rsplit("/", 1)[0] == ("" if name == "/" else name)
                        and k != name and k != "/"}
                assert {f"{'' if name == '/' else name}/{k}" for k in node.keys()} == kids


def test_group_link_limit(tmp_path):
    w = h5.Writer()
    for n in range(2 * 4 * 2 * 16 + 1):
        w.dataset(f"x{n:04d}", np.zeros(1))
    with pytest.raises(h5.H5Error, match="too many links"):
        w.write(tmp_path / "big.h5")


def test_unwritable_types_rejected():
    w = h5.Writer()
    for bad in (np.zeros(3, dtype=np.complex128), np.zeros(2, dtype=bool),
                np.zeros(2, dtype=np.float32)):
        with pytest.raises(h5.H5Error, match="cannot write element type"):
            w.dataset("bad", bad)


@pytest.mark.timeout(120)
def test_damaged_files_raise_h5error(tmp_path):
    """Random byte flips, 8-byte address overwrites and truncations of a
    written file either read or raise H5Error -- no other exception."""
    rng = np.random.default_rng(7)
    w = h5.Writer()
    w.attrs["title"] = "damaged"
    for i in range(20):
        w.dataset(f"g{i % 3}/d{i}", rng.standard_normal((3, 4)), {"k": i})
    good = tmp_path / "good.h5"
    w.write(good)
    base = good.read_bytes()

    def walk(g):
        for k in g.keys():
            x = g[k]
            walk(x) if isinstance(x, h5.Group) else x[...]
            dict(x.attrs)

    path = tmp_path / "bad.h5"
    for _ in range(600):
        b = bytearray(base)
        mode = rng.integers(3)
        if mode == 0:
            for _ in range(int(rng.integers(1, 8))):
                b[int(rng.integers(len(b)))] = int(rng.integers(256))
        elif mode == 1:
            b = b[:int(rng.integers(len(b)))]
        else:
            p = int(rng.integers(len(b) - 8))
            b[p:p + 8] = int(rng.integers(0, 2 ** 63)).to_bytes(8, "little")
        path.write_bytes(bytes(b))
        try:
            with h5.File(path) as f:
                walk(f)
        except h5.H5Error:
            pass
