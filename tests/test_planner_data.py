"""PlannerData export of a PRM roadmap (ompl_gb300/plannerdata.py): PRM::getPlannerData's vertex order,
out-edge order and component tags against the oracle's replay of PRM and PlannerData
(oracle/planner_data.py), and PlannerDataStorage's archive: a hand-spelled archive of a two-vertex
roadmap, the store/load round trip and load's rejections. Host code only (no GPU)."""
import os
import struct

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if not os.path.exists(os.path.join(ROOT, "ompl_gb300", "libgbompl.so")):
    pytest.skip("libgbompl.so not built", allow_module_level=True)

from ompl_gb300 import plannerdata as PD  # noqa: E402
from oracle.planner_data import prm_planner_data  # noqa: E402


def prm_like_edges(rng, m, k, p_valid):
    """Edges (n, m) in PRM's order: milestone m ascending, up to k distinct predecessors each."""
    src, dst = [], []
    for j in range(1, m):
        nb = rng.choice(j, size=min(k, j), replace=False)
        for n in nb:
            if rng.random() < p_valid:
                src.append(int(n))
                dst.append(j)
    return np.array(src, dtype=np.int64), np.array(dst, dtype=np.int64)


@pytest.mark.parametrize("m,k,p", [(1, 10, 1.0), (40, 3, 0.3), (500, 10, 0.2), (3000, 10, 0.05)])
def test_planner_data_matches_prm_replay(m, k, p):
    rng = np.random.default_rng(m)
    src, dst = prm_like_edges(rng, m, k, p)
    states = rng.normal(size=(m, 3))
    pd = PD.planner_data_from_edges(states, src, dst, [2, 1, 3])
    vertices, tags, out = prm_planner_data(m, list(zip(src.tolist(), dst.tolist())))
    assert pd.milestone.tolist() == vertices
    assert pd.tags.tolist() == tags
    assert [pd.targets[pd.offsets[v]:pd.offsets[v + 1]].tolist() for v in range(pd.num_vertices)] == out
    assert np.array_equal(pd.states, states[vertices])
    assert pd.num_edges == 2 * len(src) and np.all(pd.weights == 1.0)


def test_component_roots_match_disjoint_sets():
    rng = np.random.default_rng(5)
    n = 2000
    src = rng.integers(0, n, 6000)
    dst = rng.integers(0, n, 6000)
    from oracle.planner_data import DisjointSets
    ds = DisjointSets()
    for v in range(n):
        ds.make_set(v)
    for a, b in zip(src.tolist(), dst.tolist()):
        ds.union_set(a, b)
    assert PD.component_roots(src, dst, n).tolist() == [ds.find_set(v) for v in range(n)]
    with pytest.raises(Exception):
        PD.component_roots(np.array([0]), np.array([n]), n)


def test_two_vertex_archive_bytes(tmp_path):
    """Milestones 0 and 1 joined by one edge: every field of the archive spelled out."""
    states = np.array([[0.5, -1.0], [2.0, 0.25]])
    pd = PD.planner_data_from_edges(states, np.array([0]), np.array([1]), [2, 1, 2])
    path = tmp_path / "pd.bin"
    PD.store(pd, path)
    want = b"".join([
        struct.pack("<Q", 22), b"serialization::archive", struct.pack("<H", 17),
        bytes([4, 8, 4, 8]), struct.pack("<i", 1),
        struct.pack("<BI", 0, 0), struct.pack("<QQQ", 0x5044414D, 2, 2),       # Header
        struct.pack("<Q", 3), struct.pack("<3i", 2, 1, 2),                      # signature
        struct.pack("<BI", 0, 0), struct.pack("<hBI", 2, 1, 0),                 # vertex 0: class infos
        struct.pack("<Ii", 0, 1), struct.pack("<Q", 16), struct.pack("<2d", 0.5, -1.0), struct.pack("<i", 0),
        struct.pack("<h", 2), struct.pack("<Ii", 1, 1), struct.pack("<Q", 16),  # vertex 1
        struct.pack("<2d", 2.0, 0.25), struct.pack("<i", 0),
        struct.pack("<BI", 0, 0), struct.pack("<hBI", 4, 1, 0), struct.pack("<I", 2),  # edge 0 -> 1
        struct.pack("<BI", 0, 0), struct.pack("<IId", 0, 1, 1.0),
        struct.pack("<h", 4), struct.pack("<I", 3), struct.pack("<IId", 1, 0, 1.0),     # edge 1 -> 0
    ])
    assert path.read_bytes() == want


def test_store_load_round_trip_and_rejections(tmp_path):
    rng = np.random.default_rng(11)
    src, dst = prm_like_edges(rng, 800, 10, 0.15)
    states = rng.uniform(-np.pi, np.pi, size=(800, 7))
    sig = [16, 0, 7] + [2, 1] * 7
    pd = PD.planner_data_from_edges(states, src, dst, sig)
    path = tmp_path / "roadmap.pdam"
    PD.store(pd, path)
    back = PD.load(path, signature=sig)
    for f in ("states", "tags", "types", "offsets", "targets", "weights"):
        assert np.array_equal(getattr(back, f), getattr(pd, f)), f
    assert back.signature == sig
    dim, nv, ne = 7, pd.num_vertices, pd.num_edges
    fixed = 30 + 2 + 8 + 5 + 24 + 8 + 4 * len(sig)
    # first vertex: class info of the vertex data and the pointer; first edge: also the endpoint pair's
    assert os.path.getsize(path) == fixed + 10 + nv * (2 + 4 + 4 + 8 + 8 * dim + 4) + 15 + ne * 22
    with pytest.raises(ValueError, match="signature mismatch"):
        PD.load(path, signature=[2, 1, 7])
    raw = bytearray(path.read_bytes())
    bad = bytearray(raw)
    bad[30 + 2 + 8 + 5] ^= 1  # the marker's first byte
    (tmp_path / "bad").write_bytes(bad)
    with pytest.raises(ValueError, match="marker"):
        PD.load(tmp_path / "bad")
    (tmp_path / "short").write_bytes(raw[:-3])
    with pytest.raises(ValueError, match="truncated"):
        PD.load(tmp_path / "short")


def test_empty_roadmap_archive(tmp_path):
    pd = PD.planner_data_from_edges(np.zeros((4, 2)), np.zeros(0, np.int64), np.zeros(0, np.int64), [2, 1, 2])
    assert pd.num_vertices == 0 and pd.num_edges == 0
    PD.store(pd, tmp_path / "e")
    back = PD.load(tmp_path / "e")
    assert back.num_vertices == 0 and back.num_edges == 0
