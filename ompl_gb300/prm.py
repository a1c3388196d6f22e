"""Batched PRM roadmap construction on the GPU path (the caller of the path named first among the
next steps): PRM::growRoadmap + PRM::addMilestone (geometric/planners/prm/src/PRM.cpp:364-385,
570-604) with the default KStrategy (k = 10, ConnectionStrategy.h:77-81) and the default connection
filter (always true, PRM.cpp:176), done as whole batches:

  1. milestones: PRM samples with UniformValidStateSampler (sampleUniform until isValid), so the
     milestone sequence is the valid subsequence of the sampler's uniform stream, in order;
  2. neighbours: milestone m queries nearestK among the milestones added before it (nn_->add(m)
     runs after the connections, PRM.cpp:601), i.e. a prefix kNN with limit m;
  3. edges: every neighbour n is connected by checkMotion(state[n], state[m]) (PRM.cpp:590) —
     direction n -> m — and an edge is added when the motion is valid.

The edge set equals the sequential PRM's for the same sampler seed (each connection attempt is
independent of the others). Connected components are computed from the edge list on the host.

PRM* (PRM(si, starStrategy = true), PRM.cpp:226-227) connects with KStarStrategy
(ConnectionStrategy.h:120-156): milestone m asks for k(m) = ceil((e + e/d) log n) neighbours, n = m + 1
the milestone count including m (addMilestone adds the vertex before asking, PRM.cpp:574-583) and d the
state dimension. The batch runs one prefix nearestK with the largest k(m) and keeps the first k(m) of
each sorted list.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import torch

from . import base as B
from . import capi


def kstar_counts(num_milestones: int, dim: int) -> np.ndarray:
    """KStarStrategy's neighbour count for milestones 0 .. num_milestones - 1: ceil((e + e/d) log(m + 1)),
    evaluated in double precision with the C library's log, as the C++ code does. k(m) is
    non-decreasing, so each run of equal counts is located by binary search (a few hundred log calls)."""
    kc = math.e + math.e / float(dim)

    def kof(m):
        return int(math.ceil(kc * math.log(float(m + 1))))

    ks = np.empty(num_milestones, dtype=np.int64)
    m = 0
    while m < num_milestones:
        kv = kof(m)
        lo, hi = m, num_milestones - 1
        while lo < hi:
            mid = (lo + hi + 1) // 2
            if kof(mid) <= kv:
                lo = mid
            else:
                hi = mid - 1
        ks[m:lo + 1] = kv
        m = lo + 1
    return ks


@dataclass
class Roadmap:
    samples: int                 # uniform samples drawn
    milestones: torch.Tensor     # (dim, M) SoA, milestone order
    sample_index: torch.Tensor   # (M,) index of each milestone in the sample stream
    edge_src: torch.Tensor       # (E,) neighbour milestone n of each valid edge
    edge_dst: torch.Tensor       # (E,) new milestone m
    candidate_edges: int         # connection attempts (checkMotion calls)
    checked_states: int          # states the ordered DiscreteMotionValidator evaluates
    timings_ms: dict

    def adjacency_csr(self):
        """Undirected adjacency of the milestones (PRM's boost::adjacency_list<undirectedS> lists an edge
        at both ends, PRM.cpp:590-596): (offsets int64[M + 1], neighbours int64[2E]), neighbours of a
        vertex ascending."""
        m = int(self.milestones.shape[1])
        src = self.edge_src.cpu().numpy().astype(np.int64)
        dst = self.edge_dst.cpu().numpy().astype(np.int64)
        a, b = np.concatenate([src, dst]), np.concatenate([dst, src])
        order = np.lexsort((b, a))
        a, b = a[order], b[order]
        offsets = np.zeros(m + 1, dtype=np.int64)
        np.add.at(offsets, a + 1, 1)
        return np.cumsum(offsets), b

    def save(self, path):
        """Snapshot of the roadmap on the host: milestone states (one row each), their indices in the
        sample stream and the CSR adjacency, as a numpy .npz archive (Roadmap.load reads it back)."""
        offsets, neighbours = self.adjacency_csr()
        np.savez(path, states=self.milestones.T.cpu().numpy(), sample_index=self.sample_index.cpu().numpy(),
                 offsets=offsets, neighbours=neighbours, samples=np.int64(self.samples))

    @staticmethod
    def load(path):
        """The arrays Roadmap.save wrote: dict(states, sample_index, offsets, neighbours, samples)."""
        with np.load(path) as z:
            return {k: z[k] for k in z.files}


def construct_roadmap(space: B.StateSpace, checker: B.StateValidityChecker, sampler_seed: int, n_samples: int,
                      k: int = 10, schedule: int = capi.SCHEDULE_AUTO, stream=None, star: bool = False) -> Roadmap:
    """PRM's roadmap over the valid states among n_samples uniform samples: KStrategy with k neighbours,
    or KStarStrategy (PRM*) when star is set (k is then ignored)."""
    dev = torch.device("cuda")
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(6)]
    ev[0].record()
    sampler = B.StateSampler(space, sampler_seed)
    samples = sampler.sampleUniform(n_samples, soa=True, host=False, stream=stream)
    ev[1].record()
    valid = checker.isValid(samples, soa=True, stream=stream)
    sample_index = torch.nonzero(valid).squeeze(1)
    milestones = samples[:, sample_index].contiguous()
    nm = milestones.shape[1]
    ev[2].record()
    nn = B.NearestNeighborsGPU(space, capacity=max(nm, 1))
    if nm:
        nn.add(milestones, soa=True, stream=stream)
    prefix = torch.arange(nm, device=dev, dtype=torch.int64)
    if star:
        ks = torch.as_tensor(kstar_counts(nm, space.dim), device=dev)
        k = max(int(ks[-1].item()) if nm else 0, 1)
    nbr, _ = nn.nearestK(milestones, k, prefix=prefix, soa=True, want_dist=False, stream=stream)
    if star:
        nbr = torch.where(torch.arange(k, device=dev)[None, :] < ks[:, None], nbr, torch.full_like(nbr, -1))
    ev[3].record()
    dst = torch.arange(nm, device=dev, dtype=torch.int64).repeat_interleave(k)
    src = nbr.reshape(-1)
    have = src >= 0
    src, dst = src[have].contiguous(), dst[have].contiguous()
    s1 = milestones[:, src].contiguous()
    s2 = milestones[:, dst].contiguous()
    ev[4].record()
    mv = B.DiscreteMotionValidator(checker)
    r = mv.checkMotions(s1, s2, schedule=schedule, soa=True, stream=stream)
    ok = r["ok"].bool()
    fj, nd = r["first_j"].long(), r["nd"].long()
    checked = int(torch.where(fj >= 0, fj, torch.clamp(nd, min=1)).sum().item())
    ev[5].record()
    torch.cuda.synchronize()
    names = ["sample", "validity+compact", "nn add+prefix kNN", "gather", "motion"]
    timings = {n: ev[i].elapsed_time(ev[i + 1]) for i, n in enumerate(names)}
    return Roadmap(n_samples, milestones, sample_index, src[ok], dst[ok], int(src.numel()), checked, timings)


def connected_components(num_vertices: int, src: np.ndarray, dst: np.ndarray) -> int:
    """Number of connected components (PRM::uniteComponents keeps the same partition)."""
    parent = np.arange(num_vertices)

    def find(x):
        root = x
        while parent[root] != root:
            root = parent[root]
        while parent[x] != root:
            parent[x], x = root, parent[x]
        return root

    for a, b in zip(src.tolist(), dst.tolist()):
        ra, rb = find(a), find(b)
        if ra != rb:
            parent[ra] = rb
    return int(sum(1 for v in range(num_vertices) if find(v) == v))
