"""Case preparation, configuration and HDF5 I/O (no GPU).

* the HDF5 reader/writer round trip, and the reader on the reference's own
  files (FD-q rule caches, the structured sample, the prepared case) when a
  reference checkout is present;
* sample -> FD-q interpolation against the reference's prepared file
  (interpolate.py:501-585), to 1e-13 relative per component;
* config.yaml parsing and the checks of Parser.cpp:37-148;
* prepared-case (Prepare.cpp:443-687) and result-file (EigenOutput.cpp)
  writers read back by the reader, and the deterministic mode phase.
"""
from pathlib import Path

import numpy as np
import pytest

from tailor_gb300 import config, h5, output, prepare, rules
from tailor_gb300.case import Physics, make_case

from conftest import REFERENCE

REF = REFERENCE
GOLDEN = Path(__file__).resolve().parent / "golden"
needs_ref = pytest.mark.skipif(REF is None or not (REF / "case" / "config.yaml").is_file(),
                               reason="TAILOR_REFERENCE (a reference checkout) not set")


def test_writer_reader_round_trip(tmp_path):
    w = h5.Writer()
    w.attrs.update({"i": 7, "f": 2.5, "s": "k_j_dof", "u8": np.uint8(1), "neg": -3})
    a = np.arange(60.0).reshape(5, 6, 2)
    w.dataset("grid", a, {"complex": np.uint8(1)})
    w.dataset("ints", np.arange(12, dtype=np.int64).reshape(3, 4))
    for i in range(19):  # three symbol table nodes in one group
        w.dataset(f"modes/mode_{i:03d}", np.full((2, 5, 2), float(i)))
    w.group("empty")
    w.group("deep/er").dataset("x", np.array([1.0, -2.0]))
    p = tmp_path / "t.h5"
    w.write(p)
    with h5.File(p) as f:
        assert f.attrs["i"] == 7 and f.attrs["f"] == 2.5 and f.attrs["s"] == "k_j_dof"
        assert f.attrs["u8"] == 1 and f.attrs["neg"] == -3
        assert sorted(f) == ["deep", "empty", "grid", "ints", "modes"]
        assert np.array_equal(f["grid"][...], a) and f["grid"].attrs["complex"] == 1
        assert np.array_equal(f["ints"][...], np.arange(12).reshape(3, 4))
        assert list(f["modes"]) == [f"mode_{i:03d}" for i in range(19)]
        assert np.all(f["modes/mode_017"][...] == 17.0)
        assert list(f["empty"]) == []
        assert np.array_equal(f["deep/er/x"][...], [1.0, -2.0])
        with pytest.raises(KeyError):
            f["nope"]


def test_reader_rejects_non_hdf5(tmp_path):
    p = tmp_path / "x.h5"
    p.write_bytes(b"not an hdf5 file at all")
    with pytest.raises(h5.H5Error):
        h5.File(p)


@needs_ref
def test_reader_on_reference_rule_caches():
    """The reference's cached rules (fdqNodes/*.h5) read here equal the
    host generator's rules (nodes 1e-14, weights 1e-12 relative)."""
    for name, nc, q, per in (("N100_q10", 101, 10, False), ("N200_q10", 201, 10, False),
                             ("N50_q6p", 50, 6, True)):
        with h5.File(REF / "fdqNodes" / f"{name}.h5") as f:
            # N100_q10.h5 is the older schema 1 (no topology attribute)
            assert f.attrs.get("topology", "bounded") == ("periodic" if per else "bounded")
            assert int(f.attrs["node_count"]) == nc and int(f.attrs["q"]) == q
            g = rules.generate_rule(nc, q, per)
            assert np.max(np.abs(f["nodes"][...] - g.nodes)) < 1e-14
            assert np.array_equal(f["stencil_indices"][...], g.indices)
            for k in range(3):
                w = f[f"weights/d{k}"][...]
                assert np.max(np.abs(w - g.weights[k])) <= 1e-12 * np.max(np.abs(w))


@needs_ref
def test_interpolation_matches_reference_prepared_file():
    cfg = config.load_config(REF / "case" / "config.yaml")
    ours = prepare.prepare_sample(cfg.source_file, cfg.q_y, cfg.q_z, cfg.physics)
    ref = prepare.load_prepared(cfg.input_file, cfg.q_y, cfg.q_z, cfg.physics)
    assert (ours.ny, ours.nz, ours.spanwise_period) == (ref.ny, ref.nz, ref.spanwise_period)
    for a, b in ((ours.grid, ref.grid), (ours.baseflow, ref.baseflow)):
        scale = np.maximum(np.max(np.abs(b), axis=0), 1e-300)
        assert np.max(np.abs(a - b) / scale) < 1e-13
    assert np.array_equal(ours.eta.weights, ref.eta.weights)
    assert np.max(np.abs(ours.xi.nodes - ref.xi.nodes)) < 1e-14


def test_interpolation_matches_reference_prepared_fixture(tmp_path):
    """The shipped sample's source fields (a fixture read from the
    reference's sample.h5) interpolated here agree with the reference's own
    prepared fields (a fixture read from its prepared file) to 1e-13
    relative per component; no reference checkout needed."""
    src = np.load(GOLDEN / "sample_201x50_source.npz")
    prepared = np.load(GOLDEN / "sample_201x50_fields.npz")
    nz, ny = src["grid"].shape[:2]
    w = h5.Writer()
    w.attrs.update({"Ny": ny, "Nz": nz, "spanwise_periodic": 1,
                    "spanwise_period": float(src["spanwise_period"])})
    w.dataset("grid", np.stack((src["grid"], np.zeros_like(src["grid"])), axis=-1))
    w.dataset("baseflow", np.stack((src["baseflow"], np.zeros_like(src["baseflow"])), axis=-1))
    path = tmp_path / "sample.h5"
    w.write(path)
    ours = prepare.prepare_sample(path, 10, 6)
    assert (ours.ny, ours.nz) == (ny, nz)
    assert ours.spanwise_period == float(prepared["spanwise_period"])
    for a, b in ((ours.grid, prepared["grid"]), (ours.baseflow, prepared["baseflow"])):
        assert np.all(a[..., 1] == 0.0)
        scale = np.maximum(np.max(np.abs(b), axis=0), 1e-300)
        assert np.max(np.abs(a[..., 0] - b) / scale) < 1e-13


@needs_ref
def test_sample_fixture_is_the_reference_prepared_case():
    cfg = config.load_config(REF / "case" / "config.yaml")
    ref = prepare.load_prepared(cfg.input_file, cfg.q_y, cfg.q_z)
    fx = np.load(GOLDEN / "sample_201x50_fields.npz")
    assert np.array_equal(fx["grid"], ref.grid[..., 0])
    assert np.array_equal(fx["baseflow"], ref.baseflow[..., 0])
    assert float(fx["spanwise_period"]) == ref.spanwise_period


CONFIG = """CaseTitle: Sample   # comment
Folder: data
File: "sample.h5"
Q-Value:
    y: 10
    z: 6

Stability:
    Alpha:
        Real: 2.43
        Imag: 0.0
EigenSolver:
    SearchCenterOmega:
        Real: 0.3
        Imag: 0.01
    NumberOfEigenvalues: 8
    Tolerance: 1.0e-10
    MaximumIterations: 1000
Output:
    File: data/results/out.h5
Physics:
    Targets:
        ReynoldsNumber: 32500
        MachNumber: 6.0
    Gas:
        PrandtlNumber: 0.72
        GasConstant: 287.05
        RatioOfSpecificHeats: 1.4
    Transport:
        ReferenceMu: 1.716E-5       # Pa s
        ReferenceTemperature: 63.3340
        SutherlandConstant: 110.4
"""


def test_config_parse_and_paths(tmp_path):
    p = tmp_path / "config.yaml"
    p.write_text(CONFIG)
    c = config.load_config(p)
    assert c.case_title == "Sample" and (c.q_y, c.q_z) == (10, 6)
    assert c.source_file == tmp_path / "data" / "sample.h5"
    assert c.input_file == tmp_path / "data" / "FD-q" / "fdq_sample_qy10_qz6.h5"
    assert c.output_file == tmp_path / "data" / "results" / "out.h5"
    ph = c.physics
    assert (ph.reynolds, ph.mach, ph.prandtl, ph.gas_constant, ph.gamma) == \
        (32500.0, 6.0, 0.72, 287.05, 1.4)
    assert (ph.reference_viscosity, ph.reference_temperature, ph.sutherland_constant) == \
        (1.716e-5, 63.334, 110.4)
    assert ph.alpha == 2.43 and ph.omega == complex(0.3, 0.01)
    assert (ph.nev, ph.tol, ph.max_it) == (8, 1e-10, 1000)
    with pytest.raises(config.ConfigError, match="FD-q input file does not exist"):
        config.load_config(p, require_input=True)


@pytest.mark.parametrize("edit,message", [
    (("    y: 10\n", ""), "Missing YAML key: y"),
    (("        MachNumber: 6.0\n", "        MachNumber: -6.0\n"), "outside their valid ranges"),
    (("    NumberOfEigenvalues: 8\n", "    NumberOfEigenvalues: 0\n"), "must be positive"),
    (("        Real: 2.43\n", "        Real: .nan\n"), "Stability.Alpha.Real must be finite"),
    (("    y: 10\n", "    y: 1\n"), "must both be at least 2"),
    (("Output:\n    File: data/results/out.h5\n", ""), "Missing or invalid YAML mapping: Output"),
    (("Folder: data\n", "Folder: data\nFolder: other\n"), "duplicate key"),
    (("    z: 6\n", "    z: [6]\n"), "unsupported YAML construct"),
    (("    z: 6\n", "\tz: 6\n"), "tabs"),
])
def test_config_errors(tmp_path, edit, message):
    p = tmp_path / "config.yaml"
    p.write_text(CONFIG.replace(*edit))
    with pytest.raises(config.ConfigError, match=message):
        config.load_config(p)


@needs_ref
def test_reference_config():
    c = config.load_config(REF / "case" / "config.yaml", require_input=True)
    assert c.physics.reynolds == 32500 and c.physics.mach == 6.0 and c.physics.nev == 8
    assert c.input_file == REF / "case" / "data" / "FD-q" / "fdq_sample_qy10_qz6.h5"


def test_prepared_round_trip_and_checks(tmp_path):
    case = make_case(24, 16, physics=Physics())
    p = output.write_prepared(tmp_path / "fdq_x_qy10_qz6.h5", case)
    back = prepare.load_prepared(p, 10, 6)
    assert np.array_equal(back.grid, case.grid) and np.array_equal(back.baseflow, case.baseflow)
    for r0, r1 in ((case.xi, back.xi), (case.eta, back.eta)):
        assert np.array_equal(r0.nodes, r1.nodes) and np.array_equal(r0.weights, r1.weights)
        assert np.array_equal(r0.indices, r1.indices) and np.array_equal(r0.offsets, r1.offsets)
    with pytest.raises(prepare.PrepareError, match="do not match the YAML"):
        prepare.load_prepared(p, 8, 6)
    # a wrong schema version and ordering, as Prepare::readMetadata rejects them
    for key, value, msg in (("schema_version", 3, "Unsupported FD-q schema version 3"),
                            ("ordering", "j_k_dof", "ordering must be k_j_dof"),
                            ("spanwise_periodic", 0, "spanwise_periodic=1")):
        w = h5.Writer()
        with h5.File(p) as f:
            w.attrs.update(f.attrs)
            w.attrs[key] = value
            w.dataset("grid", f["grid"][...])
            w.dataset("baseflow", f["baseflow"][...])
        bad = tmp_path / f"bad_{key}.h5"
        w.write(bad)
        with pytest.raises(prepare.PrepareError, match=msg):
            prepare.load_prepared(bad)


def test_mode_phase():
    rng = np.random.default_rng(3)
    v = rng.standard_normal(50) + 1j * rng.standard_normal(50)
    m = output.fix_mode_phase(v * (2 - 3j))
    assert abs(np.linalg.norm(m) - 1) < 1e-14
    k = int(np.argmax(np.abs(m)))
    assert abs(m[k].imag) <= 1e-15 * abs(m[k]) and m[k].real > 0
    assert np.allclose(output.fix_mode_phase(1j * v), m)  # phase-independent
    with pytest.raises(ValueError):
        output.fix_mode_phase(np.zeros(4))


def test_eigen_output_schema(tmp_path):
    case = make_case(24, 16, physics=Physics(alpha=1.2, omega=complex(0.3, 0.01)))
    lam = np.array([0.01 - 0.3j, 0.02 - 0.25j])
    rng = np.random.default_rng(0)
    modes = rng.standard_normal((2, 5 * case.nodes)) + 1j * rng.standard_normal((2, 5 * case.nodes))
    p = output.write_eigen_output(tmp_path / "r" / "out.h5", case, "T", lam, [1e-12, 2e-12],
                                  modes, 8, complex(0.01, -0.3))
    with h5.File(p) as f:
        a = f.attrs
        assert a["schema_version"] == 1 and a["case"] == "T" and a["ordering"] == "k_j_dof"
        assert a["converged_modes"] == 2 and a["requested_modes"] == 8
        assert a["lambda_convention"] == "lambda=-i*omega; A_bc*q=lambda*B_bc*q"
        assert (a["search_center_lambda_real"], a["search_center_lambda_imag"]) == (0.01, -0.3)
        sl = f["spectrum/lambda"][...]
        assert np.array_equal(sl[:, 0] + 1j * sl[:, 1], lam)
        so = f["spectrum/omega"][...]
        assert np.allclose(so[:, 0] + 1j * so[:, 1], 1j * lam)
        m0 = f["modes/mode_000"][...]
        assert m0.shape == (case.nodes, 5, 2)
        mc = (m0[..., 0] + 1j * m0[..., 1]).reshape(-1)
        assert np.allclose(mc, output.fix_mode_phase(modes[0]))
        assert np.array_equal(f["grid"][...], case.grid)


# ---- the reference's interpolation and preparation tests
# (tests/Python/test_interpolate.py:77-176), restated

def test_periodic_complex_field_and_affine_translation():
    z_old = -1.0 + 2.0 * np.arange(24) / 24
    y_old = np.linspace(-1.0, 1.0, 9)
    zg, yg = np.meshgrid(z_old, y_old, indexing="ij")
    tr = 7.5

    def field(z, y):
        return (np.sin(np.pi * z) * (1.0 + y ** 3) + 1j * np.cos(2.0 * np.pi * z) * (2.0 - y)
                + 0.5 * (z + 1.0) * tr)

    z_new = -1.0 + 2.0 * np.arange(48) / 48
    y_new = np.linspace(-1.0, 1.0, 13)
    got = prepare.tensor_interpolate(z_old, y_old, field(zg, yg), z_new, y_new, shift=tr)
    zt, yt = np.meshgrid(z_new, y_new, indexing="ij")
    np.testing.assert_allclose(got, field(zt, yt), rtol=2e-6, atol=5e-6)


def test_periodic_spline_rejections():
    y = np.linspace(-1.0, 1.0, 8)
    z = np.linspace(-1.0, 1.0, 12)  # repeats the periodic endpoint
    with pytest.raises(prepare.PrepareError, match="repeat the wrap-around node"):
        prepare.tensor_interpolate(z, y, np.zeros((12, 8)), z[:-1], y)
    zu = np.array([-1.0, -0.7, -0.5, 0.0, 0.2, 0.5, 0.7])
    with pytest.raises(prepare.PrepareError, match="not uniformly spaced"):
        prepare.tensor_interpolate(zu, y, np.zeros((7, 8)), zu, y)
    zp = -1.0 + 2.0 * np.arange(5) / 5
    with pytest.raises(prepare.PrepareError, match="6 or more source nodes"):
        prepare.tensor_interpolate(zp, y, np.zeros((5, 8)), zp, y)
    zp = -1.0 + 2.0 * np.arange(12) / 12
    with pytest.raises(prepare.PrepareError, match="the source grid needs"):
        prepare.tensor_interpolate(zp, y, np.zeros((8, 12)), zp, y)


def _write_source(path, ny=8, nz=12, period=6.0):
    y = np.linspace(-1.0, 1.0, ny)
    eta = -1.0 + 2.0 * np.arange(nz) / nz
    eg, yg = np.meshgrid(eta, y, indexing="ij")
    grid = np.zeros((nz, ny, 3), dtype=np.complex128)
    grid[..., 1] = yg
    grid[..., 2] = 0.5 * (eg + 1.0) * period
    base = np.zeros((nz, ny, 5), dtype=np.complex128)
    base[..., 0] = 1.0 + 0.02 * np.cos(np.pi * eg)
    base[..., 1] = 0.5 + 0.1 * (1.0 + yg)
    base[..., 2] = 0.01 * np.sin(np.pi * eg)
    base[..., 3] = 0.02 * np.cos(np.pi * eg)
    base[..., 4] = 1.0 + 0.05 * yg
    w = h5.Writer()
    w.attrs.update({"Ny": ny, "Nz": nz, "spanwise_periodic": 1, "spanwise_period": period})
    w.dataset("grid", np.stack((grid.real, grid.imag), axis=-1))
    w.dataset("baseflow", np.stack((base.real, base.imag), axis=-1))
    w.write(path)
    return grid, base


def test_schema_v2_preparation_and_stale_cache_rebuild(tmp_path):
    from tailor_gb300 import run
    data = tmp_path / "data"
    data.mkdir()
    grid, base = _write_source(data / "sample.h5")
    (tmp_path / "config.yaml").write_text(
        CONFIG.replace("    y: 10\n    z: 6\n", "    y: 4\n    z: 4\n"))
    cfg = config.load_config(tmp_path / "config.yaml")
    case = run.prepared_case(cfg, verbose=False)
    assert (case.ny, case.nz, case.qy, case.qz) == (8, 12, 4, 4)
    with h5.File(cfg.input_file) as f:
        assert f.attrs["schema_version"] == 2 and f.attrs["source_file"] == "sample.h5"
        assert f.attrs["interpolation_version"] == 3
        assert f["discretization/z"].attrs["topology"] == "periodic"
        assert f["discretization/z/stencil_offsets"][...].shape == (12, 5)
    # corner preservation: the source's corner values survive interpolation
    g = (case.grid[..., 0] + 1j * case.grid[..., 1]).reshape(12, 8, 3)
    assert np.allclose(g[0, 0], grid[0, 0]) and np.allclose(g[-1, -1], grid[-1, -1])
    # a stale cache (wrong schema) is rebuilt
    w = h5.Writer()
    with h5.File(cfg.input_file) as f:
        w.attrs.update(f.attrs)
        w.attrs["schema_version"] = 1
    w.write(cfg.input_file)
    run.prepared_case(cfg, verbose=False)
    with h5.File(cfg.input_file) as f:
        assert f.attrs["schema_version"] == 2


def test_launcher_prepare_only(tmp_path):
    from tailor_gb300 import run
    data = tmp_path / "data"
    data.mkdir()
    _write_source(data / "sample.h5")
    (tmp_path / "config.yaml").write_text(
        CONFIG.replace("    y: 10\n    z: 6\n", "    y: 4\n    z: 4\n"))
    assert run.main(["-c", str(tmp_path / "config.yaml"), "--prepare-only"]) == 0
    assert (data / "FD-q" / "fdq_sample_qy4_qz4.h5").is_file()
    (tmp_path / "bad.yaml").write_text(CONFIG.replace("Q-Value:\n    y: 10\n    z: 6\n",
                                                      "Q-Value: 5\n"))
    assert run.main(["-c", str(tmp_path / "bad.yaml"), "--prepare-only"]) == 1


# ---- malformed prepared files (tests/CPlusPlus/test_fdq_loader_failures.py:37-72)

def _copy_with(src, dst, mutate):
    """Copy a prepared file through the writer, letting mutate(attrs, data)
    change root attributes and datasets (paths -> arrays; None removes)."""
    with h5.File(src) as f:
        attrs = dict(f.attrs)
        data = {}

        def walk(g, pre):
            for k in g:
                o = g[k]
                if isinstance(o, h5.Group):
                    walk(o, f"{pre}{k}/")
                else:
                    data[f"{pre}{k}"] = (o[...], dict(o.attrs))
        walk(f, "")
        gattrs = {p: dict(f[p].attrs) for p in ("discretization/y", "discretization/z")}
    mutate(attrs, data)
    w = h5.Writer()
    w.attrs.update(attrs)
    for path, (arr, a) in data.items():
        if arr is not None:
            w.dataset(path, arr, a)
    for p, a in gattrs.items():
        w.group(p).attrs.update(a)
    w.write(dst)


def _drop(path):
    return lambda attrs, data: data.__setitem__(path, (None, {}))


def _wrong_q(attrs, data):
    attrs["q_y"] = int(attrs["q_y"]) - 1


def _wrong_shape(attrs, data):
    a, at = data["discretization/y/weights/d2"]
    data["discretization/y/weights/d2"] = (a[:, :-1], at)


def _bad_index(attrs, data):
    a, at = data["discretization/y/stencil_indices"]
    a = a.copy()
    a[0, 0] = int(attrs["Ny"])
    data["discretization/y/stencil_indices"] = (a, at)


def _nan_weight(attrs, data):
    a, at = data["discretization/y/weights/d1"]
    a = a.copy()
    a[0, 0] = np.nan
    data["discretization/y/weights/d1"] = (a, at)


@pytest.mark.parametrize("mutate,message", [
    (_drop("discretization/y/weights/d1"), "Missing HDF5 dataset"),
    (_wrong_q, "do not match the YAML configuration"),
    (_wrong_shape, "Unexpected shape for HDF5 dataset"),
    (_bad_index, "out-of-range index"),
    (_nan_weight, "weight is not finite"),
], ids=["missing_weight", "wrong_q", "wrong_shape", "out_of_range_index", "non_finite_weight"])
def test_malformed_prepared_file(tmp_path, mutate, message):
    case = make_case(24, 16, physics=Physics())
    good = output.write_prepared(tmp_path / "good.h5", case)
    prepare.load_prepared(good, 10, 6)  # the unmodified copy loads
    bad = tmp_path / "bad.h5"
    _copy_with(good, bad, mutate)
    with pytest.raises(prepare.PrepareError, match=message):
        prepare.load_prepared(bad, 10, 6)


def test_bounded_quintic_spline_polynomial_exactness():
    """The not-a-knot quintic operator reproduces degree-5 tensor
    polynomials (the reference's bounded-spline test,
    tests/Python/test_interpolate.py:23-47, 8e-14), and agrees with
    SciPy's interpolating spline in the same space to rounding."""
    from scipy.interpolate import make_interp_spline
    from tailor_gb300 import spline
    z_old = np.linspace(-1.0, 1.0, 8)
    y_old = np.linspace(-1.0, 1.0, 9)
    zg, yg = np.meshgrid(z_old, y_old, indexing="ij")

    def f(z, y):
        return (1 + 2j) * z ** 5 + (2 - 3j) * y ** 4 + z ** 2 * y ** 3

    z_new = np.sort(np.linspace(-1.0, 1.0, 13) ** 3)
    y_new = np.sort(np.linspace(-1.0, 1.0, 14) ** 3)
    got = spline.tensor_apply(spline.bounded_matrix(z_old, z_new), f(zg, yg),
                              spline.bounded_matrix(y_old, y_new))
    zt, yt = np.meshgrid(z_new, y_new, indexing="ij")
    np.testing.assert_allclose(got, f(zt, yt), rtol=0.0, atol=8e-14)
    rng = np.random.default_rng(3)
    x = np.sort(rng.uniform(-1.0, 1.0, 40))
    v = rng.standard_normal((40, 3))
    xn = np.linspace(x[0], x[-1], 97)
    ref = make_interp_spline(x, v, k=5, axis=0)(xn)
    assert np.max(np.abs(spline.bounded_matrix(x, xn) @ v - ref)) < 1e-12 * np.max(np.abs(ref))
    with pytest.raises(spline.SplineError, match="6 or more"):
        spline.bounded_matrix(np.linspace(-1, 1, 5), [-1.0, 1.0])
    with pytest.raises(spline.SplineError, match="increase strictly"):
        spline.bounded_matrix(np.array([0.0, 1.0, 1.0, 2.0, 3.0, 4.0]), [0.5])


def test_periodic_quintic_operator_matches_the_periodic_spline():
    """The circulant periodic operator equals SciPy's periodic quintic
    interpolating spline on uniform nodes, and is exact at the nodes."""
    from scipy.interpolate import make_interp_spline
    from tailor_gb300 import spline
    rng = np.random.default_rng(5)
    for n in (6, 7, 32, 50):
        v = rng.standard_normal((n, 2))
        ph = rng.uniform(-1.5, 2.5, 41)
        x = np.arange(n + 1) / n
        ref = make_interp_spline(x, np.concatenate((v, v[:1])), k=5, bc_type="periodic",
                                 axis=0)(np.mod(ph, 1.0))
        w = spline.periodic_matrix(n, ph)
        assert np.max(np.abs(w @ v - ref)) < 1e-13 * np.max(np.abs(ref))
        assert np.max(np.abs(spline.periodic_matrix(n, np.arange(n) / n) - np.eye(n))) < 1e-14


def test_stage_report_format(tmp_path):
    """The launcher prints the reference driver's report (Process.cpp:62-176),
    in the lines its tests parse (test_metrics.py:167-184)."""
    from tailor_gb300 import run
    p = tmp_path / "config.yaml"
    p.write_text(CONFIG)
    cfg = config.load_config(p)
    case = make_case(24, 16, physics=cfg.physics)
    stages = {"metrics": {"min_jacobian": 0.5, "max_jacobian": 2.25, "max_grid_imaginary": 0.0,
                          "norms": [float(i) for i in range(10)]},
              "derivatives": {"max_baseflow_imaginary": 0.0,
                              "norms": [0.1 * i for i in range(25)]},
              "operator": {"rows": 1920, "columns": 1920, "block_size": 5,
                           "mass_used_blocks": 384.0, "mass_allocated_blocks": 384.0,
                           "spatial_used_blocks": 29568.0, "spatial_allocated_blocks": 29568.0,
                           "mass_frobenius_norm": 12.5, "spatial_frobenius_norm": 1e4},
              "bc": {"wall_nodes": 16, "farfield_nodes": 16, "incoming_modes": 16,
                     "neutral_modes": 48, "min_incoming_per_node": 1, "max_incoming_per_node": 1,
                     "max_characteristic_imaginary": 0.0, "max_eigenvector_condition": 3.5,
                     "eigen_frobenius_norm": 1e4, "eigen_mass_frobenius_norm": 12.0}}
    text = run.report(cfg, case, stages).splitlines()
    assert text[0] == "Prepared case 'Sample'"
    assert "  Ny x Nz: 24 x 16" in text
    assert "  Jacobian range: [0.5, 2.25]" in text
    assert "  metric norm eta_yz: 9" in text
    assert "  base-flow derivative norm dyz: 2 2.1 2.2 2.3 2.4" in text
    assert "  FD-q degrees: y=10, z=6; DMDA stencil width: 10" in text
    assert "  far-field incoming modes=16 (per node 1..1), neutral modes=48" in text
    d = {"requested": 8, "converged": 8, "iterations": 5, "target_re": 0.0, "target_im": -0.0,
         "max_relative_error": 3e-11}
    assert run.solve_report(d, "x.h5", 8).splitlines()[0] == \
        "  eigensolver: requested=8, converged=8, iterations=5"


def test_reader_reports_damaged_files(tmp_path):
    """Truncated or overwritten files raise H5Error (or KeyError for a name
    that is gone), never an internal parser error."""
    case = make_case(24, 16, physics=Physics())
    good = output.write_prepared(tmp_path / "good.h5", case).read_bytes()
    rng = np.random.default_rng(1)
    cuts = sorted(set([96, 200, 400, len(good) // 3, len(good) // 2, len(good) - 64]))
    for i, cut in enumerate(cuts):
        for kind in ("truncate", "scribble"):
            data = bytearray(good[:cut]) if kind == "truncate" else bytearray(good)
            if kind == "scribble":
                data[cut:cut + 64] = rng.integers(0, 256, 64, dtype=np.uint8).tobytes()
            p = tmp_path / f"bad_{i}_{kind}.h5"
            p.write_bytes(bytes(data))
            try:
                with h5.File(p) as f:
                    for name in ("grid", "baseflow", "discretization/y/weights/d1"):
                        f[name][...]
            except (h5.H5Error, KeyError):
                pass
