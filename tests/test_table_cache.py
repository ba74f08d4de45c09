"""Table-cache files (GB300TableCacheWrite / GB300TableCacheOpen): exact round trip of every
array of a serving topology, and rejection of corrupt, truncated or foreign files.  Host code
only (no GPU)."""
import os

import numpy as np
import pytest

from gpu_util import serving_bases


@pytest.fixture(scope="module")
def topo():
    from opensubdiv_gb300 import workloads
    return workloads.serving_pool(serving_bases(), n_topologies=2, cv_min=400, cv_max=1500, seed=77)[1]


def _write(tmp_path, t, limit=True):
    from opensubdiv_gb300 import server
    p = tmp_path / "t.gbtc"
    server.write_table_cache(p, t["num_control"], t["length"], t["refine"],
                             t["limit"] if limit else None)
    return p


def test_round_trip_is_exact(tmp_path, topo):
    from opensubdiv_gb300 import server
    p = _write(tmp_path, topo)
    assert not os.path.exists(str(p) + ".tmp")
    nc, L, r, lm = server.read_table_cache(p)
    assert (nc, L) == (topo["num_control"], topo["length"])
    for k, v in topo["refine"].items():
        assert np.array_equal(r[k], v), k
    for k in ("pp_sizes", "pp_offsets", "pp_indices", "pp_weights", "arrays", "patch_indices",
              "params"):
        assert np.array_equal(lm[k], np.asarray(topo["limit"][k])), k
    assert lm["triangular"] == bool(topo["limit"]["triangular"])
    # refine-only topologies carry no limit tables
    p2 = _write(tmp_path, topo, limit=False)
    assert server.read_table_cache(p2)[3] is None


def test_corrupt_truncated_and_foreign_files_are_rejected(tmp_path, topo):
    from opensubdiv_gb300 import server
    from opensubdiv_gb300._lib import GB300Error, last_error
    p = _write(tmp_path, topo)
    data = bytearray(p.read_bytes())
    bad = tmp_path / "bad.gbtc"
    data[len(data) // 2] ^= 0x40  # one flipped bit in the payload
    bad.write_bytes(bytes(data))
    with pytest.raises(GB300Error):
        server.read_table_cache(bad)
    assert "checksum" in last_error()
    server.read_table_cache(bad, verify=False)  # the structure itself is intact
    bad.write_bytes(p.read_bytes()[: len(data) - 1000])
    with pytest.raises(GB300Error):
        server.read_table_cache(bad, verify=False)
    bad.write_bytes(b"not a table cache" * 32)
    with pytest.raises(GB300Error):
        server.read_table_cache(bad)
    with pytest.raises(GB300Error):
        server.read_table_cache(tmp_path / "missing.gbtc")
