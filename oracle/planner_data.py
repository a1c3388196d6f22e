"""ORACLE (test infrastructure only): PRM::getPlannerData restated with plain Python containers.

The roadmap's edges are replayed one at a time the way OMPL builds the structures:
  * PRM::addMilestone / uniteComponents (src/ompl/geometric/planners/prm/src/PRM.cpp:570-609) with
    boost::disjoint_sets: make_set, union_set(n, m) = link(find_set(n), find_set(m)) by rank (the root
    of higher rank adopts the other; on equal ranks the second root adopts the first and its rank
    grows), find_set with path compression;
  * PRM::getPlannerData (PRM.cpp:729-756): addEdge(n, m) then addEdge(m, n), PlannerData::addVertex
    numbering vertices by first appearance and addEdge appending to the source's out-edge list unless the
    edge exists (PlannerData.cpp:383-463), every vertex tagged find_set of its milestone.
Small inputs only (pure Python loops). Only tests/ may import this module.
"""
from __future__ import annotations


class DisjointSets:
    """boost::disjoint_sets with rank and full path compression."""

    def __init__(self):
        self.parent = {}
        self.rank = {}

    def make_set(self, x):
        self.parent[x] = x
        self.rank[x] = 0

    def find_set(self, x):
        path = []
        while self.parent[x] != x:
            path.append(x)
            x = self.parent[x]
        for p in path:
            self.parent[p] = x
        return x

    def union_set(self, a, b):
        i, j = self.find_set(a), self.find_set(b)
        if i == j:
            return
        if self.rank[i] > self.rank[j]:
            self.parent[j] = i
        else:
            self.parent[i] = j
            if self.rank[i] == self.rank[j]:
                self.rank[j] += 1


def prm_planner_data(n_milestones, edges):
    """edges: [(n, m), ...] in PRM's insertion order. Returns (vertex_milestones, tags, out_edges) where
    out_edges[v] lists the target vertices of v's out-edges in insertion order."""
    ds = DisjointSets()
    for v in range(n_milestones):
        ds.make_set(v)
    for n, m in edges:
        ds.union_set(n, m)
    index, vertices, out = {}, [], []

    def add_vertex(x):
        if x not in index:
            index[x] = len(vertices)
            vertices.append(x)
            out.append([])
        return index[x]

    def add_edge(a, b):
        ia, ib = add_vertex(a), add_vertex(b)
        if ib not in out[ia]:
            out[ia].append(ib)

    for n, m in edges:
        add_edge(n, m)
        add_edge(m, n)
    tags = [ds.find_set(x) for x in vertices]
    return vertices, tags, out
