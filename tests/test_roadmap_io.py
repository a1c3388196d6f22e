"""Roadmap snapshot (ompl_gb300.prm.Roadmap): undirected CSR adjacency and the .npz round trip, on a
small hand-made roadmap, and PRM*'s neighbour counts (no GPU needed)."""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from ompl_gb300.prm import Roadmap, connected_components, kstar_counts  # noqa: E402


@pytest.mark.parametrize("dim", [1, 2, 7, 10])
def test_kstar_counts_match_the_per_milestone_formula(dim):
    # KStarStrategy (ConnectionStrategy.h:143-147): k = ceil((e + e/d) log n), n = milestones so far
    kc = math.e + math.e / dim
    want = [int(math.ceil(kc * math.log(m + 1))) for m in range(20000)]
    assert kstar_counts(20000, dim).tolist() == want
    assert kstar_counts(0, dim).size == 0 and kstar_counts(1, dim).tolist() == [0]


def _roadmap():
    states = torch.arange(10, dtype=torch.float64).reshape(2, 5)  # (dim, M) = 5 milestones in R^2
    return Roadmap(samples=9, milestones=states, sample_index=torch.tensor([0, 2, 3, 6, 8]),
                   edge_src=torch.tensor([0, 1, 0, 3]), edge_dst=torch.tensor([1, 2, 2, 4]),
                   candidate_edges=6, checked_states=17, timings_ms={})


def test_adjacency_csr_lists_each_edge_at_both_ends():
    offsets, nbrs = _roadmap().adjacency_csr()
    assert offsets.tolist() == [0, 2, 4, 6, 7, 8]
    assert [nbrs[offsets[v]:offsets[v + 1]].tolist() for v in range(5)] == [[1, 2], [0, 2], [0, 1], [4], [3]]
    assert connected_components(5, np.array([0, 1, 0, 3]), np.array([1, 2, 2, 4])) == 2


def test_save_load_round_trip(tmp_path):
    r = _roadmap()
    p = tmp_path / "roadmap.npz"
    r.save(p)
    z = Roadmap.load(p)
    assert np.array_equal(z["states"], r.milestones.T.numpy())
    assert z["sample_index"].tolist() == [0, 2, 3, 6, 8] and int(z["samples"]) == 9
    off, nb = r.adjacency_csr()
    assert np.array_equal(z["offsets"], off) and np.array_equal(z["neighbours"], nb)
