"""Physics tables (the "dxmcg-physics 1" text format): the engine's host library and
the oracle read the same file, and today's parametric model written as a table
(opendxmc_gb300/data/physics_model.txt) reproduces the model.  No GPU."""
import numpy as np
import pytest

from opendxmc_gb300 import phantoms as P

ROOT_DATA = __import__("pathlib").Path(__file__).resolve().parents[1] / "opendxmc_gb300" / "data"
MODEL_TABLE = ROOT_DATA / "physics_model.txt"
GRID = 1.0 + 0.5 * np.arange(300)
OFF_GRID = np.array([1.3, 4.2, 4.04, 8.73, 33.17, 69.6, 88.1, 149.9, 150.7])
MATERIALS = [P.WATER, P.BONE, P.LUNG, P.AIR, P.ADIPOSE, {53: 1.0}, {74: 1.0}]


@pytest.fixture
def tables(engine, oracle):
    """Both sides back on the model after each test (the tables are process-wide)."""
    yield engine, oracle
    engine.physics_reset()
    oracle.physics_reset()


def attenuations(mod, zw, E, correction):
    return np.stack(mod.attenuation(zw, E, correction))


def modified_table(src, dst):
    """The model's table with oxygen's photoelectric cross section x 1.5, hydrogen's
    form-factor scale x 2, calcium's K edge moved, and an unfiltered 100 kVp tube."""
    out = []
    z = None
    for line in src.read_text().splitlines():
        w = line.split()
        if w and w[0] == "element":
            z = int(w[1])
        if z == 8 and w and w[0] == "photo":
            line = "  photo " + " ".join(repr(float(v) * 1.5) for v in w[1:])
        if z == 1 and w and w[0] == "formfactor":
            line = f"  formfactor {float(w[1]) * 2.0!r}"
        if z == 20 and w and w[0] == "edges":
            line = f"  edges 4.5 {w[2]}"
        out.append(line)
    E = np.arange(1.0, 101.0)
    out.append("tube 100 12 100 " + " ".join(f"{float(e)!r} {float(np.exp(-((e - 45.0) / 20.0) ** 2))!r}" for e in E))
    dst.write_text("\n".join(out) + "\n")


def test_model_table_reproduces_the_model(tables, tmp_path):
    engine, oracle = tables
    ref = {(i, c): attenuations(engine, zw, GRID, c) for i, zw in enumerate(MATERIALS) for c in (0, 1, 2)}
    spec = engine.tube_spectrum(120.0, {13: 6.0})
    # written here and now: bit for bit on the table grid
    fresh = tmp_path / "model.txt"
    zs = sorted({z for m in MATERIALS for z in m} | {13})
    engine.physics_write(fresh, zs)
    engine.physics_load(fresh)
    for (i, c), a in ref.items():
        np.testing.assert_array_equal(attenuations(engine, MATERIALS[i], GRID, c), a)
    e2, w2 = engine.tube_spectrum(120.0, {13: 6.0})
    np.testing.assert_array_equal(w2, spec[1])
    # the committed model table (written on another machine's libm): within 1e-13
    engine.physics_load(MODEL_TABLE)
    for (i, c), a in ref.items():
        np.testing.assert_allclose(attenuations(engine, MATERIALS[i], GRID, c), a, rtol=1e-13, atol=0)
    engine.physics_reset()
    for (i, c), a in ref.items():
        np.testing.assert_array_equal(attenuations(engine, MATERIALS[i], GRID, c), a)


@pytest.mark.parametrize("which", ["model", "modified"])
def test_library_and_oracle_read_tables_alike(tables, tmp_path, which):
    engine, oracle = tables
    path = MODEL_TABLE
    if which == "modified":
        path = tmp_path / "modified.txt"
        modified_table(MODEL_TABLE, path)
    base = [attenuations(engine, zw, OFF_GRID, 1) for zw in MATERIALS]
    engine.physics_load(path)
    oracle.physics_load(path)
    for zw in MATERIALS:
        for c in (0, 1, 2):
            for E in (GRID, OFF_GRID):
                np.testing.assert_allclose(attenuations(engine, zw, E, c), attenuations(oracle, zw, E, c),
                                           rtol=1e-13, atol=0)
    for kvp, filt in ((100.0, {13: 2.5}), (120.0, {13: 6.0}), (80.0, {})):
        e1, w1 = oracle.tube_spectrum(kvp, filt)
        e2, w2 = engine.tube_spectrum(kvp, filt)
        np.testing.assert_array_equal(e1, e2)
        np.testing.assert_allclose(w2, w1, rtol=1e-13, atol=1e-300)
    if which == "modified":
        water = attenuations(engine, P.WATER, OFF_GRID, 1)
        assert np.all(water[0] > 1.2 * base[0][0])  # oxygen's photoelectric x 1.5
        E, w = engine.tube_spectrum(100.0, {13: 2.5})
        assert E[np.argmax(w)] > 40.0  # the loaded Gaussian-shaped tube, not Kramers' law
        for s in (oracle, engine):
            assert s.tube_mean_energy(100.0, {13: 2.5}) == pytest.approx(
                engine.tube_mean_energy(100.0, {13: 2.5}), rel=1e-13)


@pytest.mark.parametrize("text", [
    "dxmcg-physics 2\n",
    "dxmcg-physics 1\nelement 8 16.0\nend\n",
    "dxmcg-physics 1\nenergies 3 1 2 1.5\n",
    "dxmcg-physics 1\nenergies 2 1 2\nelement 8 16.0\n  photo 1 2\n  incoherent 1 2\n  coherent 1 -2\n"
    "  formfactor 1\n  edges 0.5 0\n  fluorescence 0.4 0.01\n  shells 1 2 0.5 0.01\nend\n",
    "dxmcg-physics 1\nenergies 2 1 2\nbogus 3\n",
])
def test_malformed_tables_are_refused(tables, tmp_path, text):
    engine, oracle = tables
    path = tmp_path / "bad.txt"
    path.write_text(text)
    ref = attenuations(engine, P.WATER, GRID, 1)
    with pytest.raises(Exception):
        engine.physics_load(path)
    with pytest.raises(ValueError):
        oracle.physics_load(path)
    np.testing.assert_array_equal(attenuations(engine, P.WATER, GRID, 1), ref)
