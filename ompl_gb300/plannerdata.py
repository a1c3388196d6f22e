"""A PRM roadmap as OMPL PlannerData, and PlannerDataStorage's archive of it.

`planner_data(roadmap, space)` is PRM::getPlannerData (src/ompl/geometric/planners/prm/src/PRM.cpp:729-756)
for a roadmap without start or goal states: for every roadmap edge (n, m) in the order PRM added it
(milestone m ascending, its neighbours in nearestK order, PRM.cpp:585-597) it adds the edge n -> m and the
reverse edge m -> n (PlannerData::addEdge, PlannerData.cpp:424-463: vertices numbered by first
appearance, each vertex's out-edges kept in insertion order, weight Cost(1.0)), and tags both vertices
with their component representative `disjointSets_.find_set` (gbo_prm_component_roots). Milestones
without edges are not vertices of the planner data, as in PRM.

`store(pd, path)` writes what PlannerDataStorage::store writes (PlannerDataStorage.cpp:55-90,
PlannerDataStorage.h:107-287): a Header {marker 0x5044414D "PDAM", vertex count, edge count, the state
space signature (StateSpace::computeSignature, StateSpace.cpp:219-224: [length, type, dimension])}, then
every vertex {PlannerDataVertex pointer (its tag), the serialized state (the state's doubles, as
RealVectorStateSpace::serialize and SO2StateSpace::serialize copy them), the vertex type 0 standard /
1 start / 2 goal}, then every edge by source vertex and out-edge order {PlannerDataEdge pointer,
(source, target), weight}.
The bytes follow the layout of a Boost.Serialization binary_oarchive (library version 17, LP64,
little-endian) as Boost's archive sources define it:

  preamble   u64 22, "serialization::archive", u16 library version, u8 sizeof(int)=4, sizeof(long)=8,
             sizeof(float)=4, sizeof(double)=8, i32 1
  class info the first object of each class saved by value: u8 tracking (0), u32 version (0); classes
             numbered in the order first met: Header 0, vertex data 1, PlannerDataVertex 2, edge data 3,
             PlannerDataEdge 4, std::pair<unsigned, unsigned> 5
  pointer    first of its class: i16 class id, u8 tracking (1), u32 version (0); later: i16 class id;
             then u32 object id (objects numbered in saving order) and the object's fields
  vector     u64 count, then the elements' bytes (vectors of primitives carry no class info)
  enum       i32; uint_fast32_t marker and size_t counts u64; unsigned u32; double f64

Boost is not available to write a reference archive, so this layout is not checked against one: `load`
reads exactly this layout back (and rejects anything else), and the tests check the round trip and the
PRM order, tags and edge lists against the oracle's PRM roadmap.
"""
from __future__ import annotations

import ctypes as C
import struct
from dataclasses import dataclass

import numpy as np

from . import capi
from .capi import check, lib

MARKER = 0x5044414D
SIGNATURE_TEXT = b"serialization::archive"
LIBRARY_VERSION = 17
STANDARD, START, GOAL = 0, 1, 2
_CLASS_HEADER, _CLASS_VERTEX_DATA, _CLASS_VERTEX, _CLASS_EDGE_DATA, _CLASS_EDGE, _CLASS_PAIR = range(6)
_SPACE_TYPES = {capi.SPACE_REAL_VECTOR: 1, capi.SPACE_KINEMATIC_CHAIN: 1, capi.SPACE_SO2: 2}


@dataclass
class PlannerData:
    """PlannerData's vertices (states, tags, types) and directed edges (out-edges of each vertex in
    insertion order: CSR offsets / targets, with their weights)."""
    states: np.ndarray       # (V, dim) float64
    tags: np.ndarray         # (V,) int32
    types: np.ndarray        # (V,) int32: STANDARD / START / GOAL
    offsets: np.ndarray      # (V + 1,) int64
    targets: np.ndarray      # (E,) int64
    weights: np.ndarray      # (E,) float64
    signature: list          # StateSpace::computeSignature
    milestone: np.ndarray = None  # (V,) roadmap milestone of each vertex (not stored in the archive)

    @property
    def num_vertices(self):
        return int(self.states.shape[0])

    @property
    def num_edges(self):
        return int(self.targets.shape[0])


def space_signature(space):
    """StateSpace::computeSignature (StateSpace.cpp:113-133, 219-224): [length, type, dimension] for
    RealVector (type 1; the chain space derives from it) and SO2 (type 2). The wrapped joint space has
    no OMPL class; its states are laid out as those of a CompoundStateSpace of `dim` SO2 spaces (type 0,
    then each subspace's type and dimension), which is the signature it gets."""
    if space.kind == capi.SPACE_WRAP_L2:
        body = [0, int(space.dim)] + [2, 1] * int(space.dim)
        return [len(body)] + body
    if space.kind not in _SPACE_TYPES:
        raise ValueError("no state space signature for this space")
    return [2, _SPACE_TYPES[space.kind], int(space.dim)]


def component_roots(src, dst, n_vertices):
    """disjointSets_.find_set of every milestone after PRM's unions (gbo_prm_component_roots)."""
    src = np.ascontiguousarray(src, dtype=np.int64)
    dst = np.ascontiguousarray(dst, dtype=np.int64)
    root = np.empty(n_vertices, dtype=np.int64)
    check(lib().gbo_prm_component_roots(src.ctypes.data_as(C.c_void_p), dst.ctypes.data_as(C.c_void_p),
                                        int(src.size), int(n_vertices), root.ctypes.data_as(C.c_void_p)))
    return root


def planner_data(roadmap, space):
    """PRM::getPlannerData of a roadmap (prm.Roadmap) over `space`."""
    states = roadmap.milestones.T.cpu().numpy().astype(np.float64)
    src = roadmap.edge_src.cpu().numpy().astype(np.int64)
    dst = roadmap.edge_dst.cpu().numpy().astype(np.int64)
    return planner_data_from_edges(states, src, dst, space_signature(space))


def planner_data_from_edges(states, src, dst, signature):
    """PlannerData of milestones `states` and edges (src[e], dst[e]) in PRM's insertion order."""
    nm = states.shape[0]
    roots = component_roots(src, dst, nm)
    seq = np.empty(2 * src.size, dtype=np.int64)  # the vertex sequence addEdge meets: n0, m0, n1, m1, ...
    seq[0::2], seq[1::2] = src, dst
    uniq, first = np.unique(seq, return_index=True)
    milestone = uniq[np.argsort(first, kind="stable")]  # vertex index -> milestone, by first appearance
    index = np.full(nm, -1, dtype=np.int64)
    index[milestone] = np.arange(milestone.size)
    # out-edges: the edge sequence n->m, m->n, ... grouped by source vertex, insertion order kept
    frm = np.empty_like(seq)
    to = np.empty_like(seq)
    frm[0::2], to[0::2] = index[src], index[dst]
    frm[1::2], to[1::2] = index[dst], index[src]
    order = np.argsort(frm, kind="stable")
    nv = milestone.size
    offsets = np.zeros(nv + 1, dtype=np.int64)
    np.add.at(offsets, frm + 1, 1)
    return PlannerData(states=states[milestone].copy(), tags=roots[milestone].astype(np.int32),
                       types=np.zeros(nv, dtype=np.int32), offsets=np.cumsum(offsets), targets=to[order],
                       weights=np.ones(seq.size, dtype=np.float64), signature=list(signature),
                       milestone=milestone)


def _preamble():
    return (struct.pack("<Q", len(SIGNATURE_TEXT)) + SIGNATURE_TEXT + struct.pack("<H", LIBRARY_VERSION) +
            struct.pack("<BBBBi", 4, 8, 4, 8, 1))


def _vertex_dtype(dim):
    return np.dtype([("cid", "<i2"), ("oid", "<u4"), ("tag", "<i4"), ("nb", "<u8"), ("x", "<f8", (dim,)),
                     ("type", "<i4")])


_EDGE_DTYPE = np.dtype([("cid", "<i2"), ("oid", "<u4"), ("frm", "<u4"), ("to", "<u4"), ("w", "<f8")])
_CLASS_INFO = struct.pack("<BI", 0, 0)


def store(pd: PlannerData, path):
    """PlannerDataStorage::store(pd, filename) in the layout above."""
    nv, ne, dim = pd.num_vertices, pd.num_edges, pd.states.shape[1]
    if len(pd.signature) < 3 or pd.signature[0] != len(pd.signature) - 1 or pd.signature[2] != dim:
        raise ValueError("signature does not match the states' dimension")
    out = bytearray(_preamble())
    out += _CLASS_INFO + struct.pack("<QQQ", MARKER, nv, ne)
    out += struct.pack("<Q", len(pd.signature)) + np.asarray(pd.signature, dtype="<i4").tobytes()
    vd = _vertex_dtype(dim)
    verts = np.zeros(nv, dtype=vd)
    verts["cid"], verts["oid"], verts["tag"] = _CLASS_VERTEX, np.arange(nv), pd.tags
    verts["nb"], verts["x"], verts["type"] = 8 * dim, pd.states, pd.types
    vb = verts.tobytes()
    if nv:
        # the first vertex record carries the class info of the vertex data and of PlannerDataVertex
        out += _CLASS_INFO + vb[:2] + struct.pack("<BI", 1, 0) + vb[2:]
    frm = np.repeat(np.arange(nv), np.diff(pd.offsets))
    edges = np.zeros(ne, dtype=_EDGE_DTYPE)
    edges["cid"], edges["oid"], edges["frm"] = _CLASS_EDGE, nv + np.arange(ne), frm
    edges["to"], edges["w"] = pd.targets, pd.weights
    eb = edges.tobytes()
    if ne:
        # the first edge record: class info of the edge data, of PlannerDataEdge and of the endpoint pair
        out += _CLASS_INFO + eb[:2] + struct.pack("<BI", 1, 0) + eb[2:6] + _CLASS_INFO + eb[6:]
    with open(path, "wb") as f:
        f.write(out)


class _Reader:
    def __init__(self, data):
        self.b = data
        self.p = 0

    def raw(self, n):
        if self.p + n > len(self.b):
            raise ValueError("planner data archive is truncated")
        v = self.b[self.p:self.p + n]
        self.p += n
        return v

    def take(self, fmt):
        v = struct.unpack(fmt, self.raw(struct.calcsize(fmt)))
        return v if len(v) > 1 else v[0]

    def expect(self, fmt, value, what):
        got = self.take(fmt)
        if got != value:
            raise ValueError(f"planner data archive: bad {what} ({got!r}, expected {value!r})")


def load(path, signature=None):
    """PlannerDataStorage::load: the PlannerData `store` wrote. Raises ValueError on a marker or (when
    `signature` is given) a state space signature mismatch, as load returns false for them, and on
    anything this layout does not allow."""
    with open(path, "rb") as f:
        data = f.read()
    r = _Reader(data)
    r.expect("<Q", len(SIGNATURE_TEXT), "archive signature")
    if r.raw(len(SIGNATURE_TEXT)) != SIGNATURE_TEXT:
        raise ValueError("not a binary archive")
    lib_version = r.take("<H")
    if not 8 <= lib_version <= 20:
        raise ValueError(f"unsupported archive library version {lib_version}")
    r.expect("<BBBBi", (4, 8, 4, 8, 1), "primitive sizes")
    r.expect("<BI", (0, 0), "header class info")
    marker, nv, ne = r.take("<QQQ")
    if marker != MARKER:
        raise ValueError("PlannerData archive marker not found")
    ns = r.take("<Q")
    sig = [int(v) for v in np.frombuffer(r.raw(4 * ns), dtype="<i4")]
    if ns < 3 or sig[0] != ns - 1:
        raise ValueError("malformed state space signature")
    if signature is not None and list(signature) != sig:
        raise ValueError("StateSpace signature mismatch")
    dim = sig[2]
    vd = _vertex_dtype(dim)
    vb = b""
    if nv:
        r.expect("<BI", (0, 0), "vertex data class info")
        head = r.raw(2)
        r.expect("<BI", (1, 0), "PlannerDataVertex class info")
        vb = head + r.raw(vd.itemsize * nv - 2)
    verts = np.frombuffer(vb, dtype=vd, count=nv)
    eb = b""
    if ne:
        r.expect("<BI", (0, 0), "edge data class info")
        head = r.raw(2)
        r.expect("<BI", (1, 0), "PlannerDataEdge class info")
        oid = r.raw(4)
        r.expect("<BI", (0, 0), "endpoint pair class info")
        eb = head + oid + r.raw(_EDGE_DTYPE.itemsize * ne - 6)
    edges = np.frombuffer(eb, dtype=_EDGE_DTYPE, count=ne)
    if r.p != len(r.b):
        raise ValueError("trailing bytes after the last edge")
    if np.any(verts["cid"] != _CLASS_VERTEX) or np.any(edges["cid"] != _CLASS_EDGE):
        raise ValueError("unexpected class id")
    if not (np.array_equal(verts["oid"], np.arange(nv)) and np.array_equal(edges["oid"], nv + np.arange(ne))):
        raise ValueError("unexpected object ids")
    if np.any(verts["nb"] != 8 * dim):
        raise ValueError("serialized state length does not match the signature")
    frm = edges["frm"].astype(np.int64)
    if ne and (np.any(np.diff(frm) < 0) or frm[-1] >= nv or np.any(edges["to"] >= nv)):
        raise ValueError("edges are not grouped by source vertex or name a missing vertex")
    offsets = np.zeros(nv + 1, dtype=np.int64)
    np.add.at(offsets, frm + 1, 1)
    return PlannerData(states=verts["x"].reshape(nv, dim).copy(), tags=verts["tag"].astype(np.int32),
                       types=verts["type"].astype(np.int32), offsets=np.cumsum(offsets),
                       targets=edges["to"].astype(np.int64), weights=edges["w"].astype(np.float64), signature=sig)
