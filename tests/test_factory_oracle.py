"""The stencil-table factory's oracle and mask recorder against the reference.

tests/golden/factory_masks.npz holds, per case, the masks GB300MaskRecorder recorded from the
reference's Far::PrimvarRefiner and the tables Far::StencilTableFactory built from the same
refiner (tests/golden/make_golden.py).  The oracle's restatement of StencilBuilder's merge
(oracle/osd_oracle.c, orc_factory_create) must rebuild those tables bit for bit."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "factory_masks.npz")


def load_case(z, name):
    """(num_control, per-level masks) of a fixture case; each level's offsets start at 0 and
    index that level's slice of the concatenated sources / weights."""
    rows = z[f"{name}_mask_rows"]
    off = z[f"{name}_mask_offsets"]
    src, w = z[f"{name}_mask_sources"], z[f"{name}_mask_weights"]
    out, base, o = [], 0, 0
    for n in rows:
        lo = off[o:o + n + 1].astype(np.int64)
        o += n + 1
        nnz = int(lo[-1])
        out.append(dict(offsets=lo, sources=src[base:base + nnz], weights=w[base:base + nnz]))
        base += nnz
    return int(z[f"{name}_num_control"]), out


def far_table(z, name, tag):
    return {k: z[f"{name}_{tag}_{k}"] for k in ("sizes", "offsets", "indices", "weights")}


def same_table(a, b):
    for k in ("sizes", "offsets", "indices"):
        if not np.array_equal(a[k], b[k]):
            return False
    return np.array_equal(np.asarray(a["weights"], np.float32).view(np.uint32),
                          np.asarray(b["weights"], np.float32).view(np.uint32))


LIMIT = os.path.join(ROOT, "tests", "golden", "factory_limit.npz")
CHANNELS = ("weights", "du_weights", "dv_weights", "duu_weights", "duv_weights", "dvv_weights")


def cases():
    return [str(c) for c in np.load(GOLDEN)["cases"]]


def limit_cases():
    return [str(c) for c in np.load(LIMIT)["cases"]]


def limit_case(z, name):
    """The recorded inputs of one GPU LimitStencilTableFactory case as plain arrays."""
    g = lambda k, d=None: z[f"{name}_{k}"] if f"{name}_{k}" in z else d  # noqa: E731
    rows = g("level_rows")
    off, src, w = g("level_offsets"), g("level_sources"), g("level_weights")
    levels, base, o = [], 0, 0
    for n in rows:
        lo = off[o:o + n + 1].astype(np.int64)
        o += n + 1
        nnz = int(lo[-1])
        levels.append(dict(offsets=lo, sources=src[base:base + nnz], weights=w[base:base + nnz]))
        base += nnz
    nc = int(g("num_channels"))
    rec = dict(num_control=int(g("num_control")), levels=levels, num_channels=nc,
               spliced=bool(int(g("spliced"))), intermediate=bool(int(g("cv_intermediate"))),
               local=(g("local_offsets"), g("local_sources"), g("local_weights")),
               loc=(g("loc_offsets"), g("loc_sources"), [g(f"loc_w{c}") for c in range(nc)]))
    far = dict(sizes=g("far_sizes"), offsets=g("far_offsets"), indices=g("far_indices"))
    for c in range(nc):
        far[CHANNELS[c]] = g(f"far_w{c}")
    return rec, far


def same_limit_table(a, b, nc):
    for k in ("sizes", "offsets", "indices"):
        if not np.array_equal(a[k], b[k]):
            return False
    return all(np.array_equal(np.asarray(a[CHANNELS[c]], np.float32).view(np.uint32),
                              np.asarray(b[CHANNELS[c]], np.float32).view(np.uint32))
               for c in range(nc))


@pytest.mark.parametrize("name", limit_cases())
def test_oracle_limit_pipeline_rebuilds_far_limit_tables(name):
    """Refined-vertex table, local-point splice (AppendLocalPointStencilTable) and per-location
    merges from the recorded masks equal Far::LimitStencilTableFactory's table bit for bit."""
    rec, far = limit_case(np.load(LIMIT), name)
    cv = oracle.factory_create(rec["num_control"], rec["levels"], intermediate=rec["intermediate"],
                               control=True)
    if rec["spliced"]:
        o, s, w = rec["local"]
        cv = oracle.compose_rows(cv, o, s, [w], append_base=True)
    o, s, ws = rec["loc"]
    got = oracle.compose_rows(cv, o, s, ws)
    assert same_limit_table(got, far, rec["num_channels"])


@pytest.mark.parametrize("name", cases())
@pytest.mark.parametrize("tag,inter,ctrl", [("all", True, False), ("last_ctrl", False, True)])
def test_oracle_factory_rebuilds_far_tables(name, tag, inter, ctrl):
    z = np.load(GOLDEN)
    nc, levels = load_case(z, name)
    got = oracle.factory_create(nc, levels, intermediate=inter, control=ctrl)
    assert same_table(got, far_table(z, name, tag))


def test_fixture_exercises_waves_and_long_rows():
    """Catmark masks refer to same-level face points (two dependency waves), the pole case has
    rows longer than a warp's 256-entry shared list and Loop masks have no same-level refs."""
    z = np.load(GOLDEN)
    nc, levels = load_case(z, "cube")
    first = nc
    same_level = 0
    for d in levels:
        n = len(d["offsets"]) - 1
        same_level += int((d["sources"] >= first).sum())
        first += n
    assert same_level > 0
    nc, levels = load_case(z, "loop")
    first = nc
    for d in levels:
        assert not (d["sources"] >= first).any()
        first += len(d["offsets"]) - 1
    assert far_table(z, "pole", "all")["sizes"].max() > 256


def test_oracle_factory_rejects_bad_sources():
    z = np.load(GOLDEN)
    nc, levels = load_case(z, "cube")
    bad = [dict(d) for d in levels]
    bad[2] = dict(bad[2], sources=bad[2]["sources"].copy())
    bad[2]["sources"][5] = nc + 3  # a level-1 vertex named by a level-3 mask
    with pytest.raises(ValueError):
        oracle.factory_create(nc, bad)


def test_recorder_matches_fixture():
    """Re-record the masks with the reference in this container (skipped without it)."""
    import ref
    if not ref.available():
        pytest.skip("oracle/_ref/libosdref.so not built")
    from opensubdiv_gb300 import shapes
    z = np.load(GOLDEN)
    r = ref.Refiner(shapes.cube(4, noise=0.01, seed=41)).refine_uniform(3)
    nc, levels = ref.record_masks(r, ref.INTERPOLATE_VERTEX)
    nc0, want = load_case(z, "cube")
    assert nc == nc0
    for a, b in zip(levels, want):
        assert np.array_equal(a["offsets"], b["offsets"])
        assert np.array_equal(a["sources"], b["sources"])
        assert np.array_equal(a["weights"].view(np.uint32), b["weights"].view(np.uint32))


def test_factory_header_compiles_standalone():
    """Without OpenSubdiv the header provides the recorder (no Far-facing Create)."""
    src = os.path.join(ROOT, "tests", "cpp", "factory_client.cpp")
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    r = subprocess.run([gxx, "-std=c++14", "-fsyntax-only", f"-I{ROOT}/include", src],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_factory_header_compiles_with_far():
    """With the reference's headers the Far-facing GB300StencilTableFactory compiles."""
    refdir = os.environ.get("OSD_REFERENCE", "/root/reference")
    if not os.path.isdir(os.path.join(refdir, "opensubdiv", "far")):
        pytest.skip("reference headers not present")
    src = os.path.join(ROOT, "tests", "cpp", "factory_client.cpp")
    r = subprocess.run(["g++", "-std=c++14", "-fsyntax-only", "-DFACTORY_CLIENT_WITH_FAR",
                        f"-I{ROOT}/include", f"-I{refdir}", src], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
