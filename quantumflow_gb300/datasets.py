"""Standard graph sets for QAOA evaluation (quantumflow/datasets/__init__.py:23-37).

The reference ships 100 Erdos-Renyi G(n, 0.5) graphs per size n = 6..32 as
graph6 files (``datasets/data/graph{n}er100.g6``) and reads them with
networkx.  Here the graph6 format (B. McKay's published encoding: a size
prefix, then the upper triangle of the adjacency matrix column by column,
six bits per printable byte) is read and written directly into
:class:`quantumflow_gb300.qaoa.Graph`, so no graph library is needed on the
GPU host.  ``load_stdgraphs(size, path)`` reads a graph6 file set from
``path`` (for example the reference's data directory); without one it
returns a seeded synthetic set of the same shape (100 graphs of G(size, 0.5)).
"""
import os
from typing import Iterable, List, Union

from .qaoa import Graph, gnp_random_graph

__all__ = ["read_graph6", "write_graph6", "load_stdgraphs"]


def _decode_size(data: bytes):
    """n and the number of bytes its encoding takes."""
    if data[0] != 126:
        return data[0] - 63, 1
    if data[1] != 126:
        v = 0
        for b in data[1:4]:
            v = (v << 6) | (b - 63)
        return v, 4
    v = 0
    for b in data[2:8]:
        v = (v << 6) | (b - 63)
    return v, 8


def _encode_size(n: int) -> bytes:
    if n < 0:
        raise ValueError("negative graph size")
    if n <= 62:
        return bytes([n + 63])
    if n <= 258047:
        return bytes([126] + [((n >> s) & 63) + 63 for s in (12, 6, 0)])
    if n <= 68719476735:
        return bytes([126, 126] + [((n >> s) & 63) + 63 for s in (30, 24, 18, 12, 6, 0)])
    raise ValueError("graph too large for graph6")


def graph6_to_graph(line: Union[bytes, str]) -> Graph:
    """One graph6 record (no newline) as a Graph on nodes 0..n-1."""
    data = line.encode("ascii") if isinstance(line, str) else bytes(line)
    if data.startswith(b">>graph6<<"):
        data = data[10:]
    if any(b < 63 or b > 126 for b in data):
        raise ValueError("not a graph6 record")
    n, off = _decode_size(data)
    body = data[off:]
    need = (n * (n - 1) // 2 + 5) // 6
    if len(body) != need:
        raise ValueError(f"graph6 record has {len(body)} data bytes, expected {need}")
    g = Graph(nodes=range(n))
    bit = 0
    for j in range(1, n):
        for i in range(j):
            byte = body[bit // 6] - 63
            if (byte >> (5 - bit % 6)) & 1:
                g.add_edge(i, j)
            bit += 1
    return g


def graph_to_graph6(g) -> bytes:
    """A graph on nodes 0..n-1 (any object with nodes and edges()) as one
    graph6 record (no header, no newline)."""
    nodes = sorted(g.nodes)
    index = {q: k for k, q in enumerate(nodes)}
    n = len(nodes)
    adj = set()
    for u, v in g.edges():
        a, b = index[u], index[v]
        adj.add((min(a, b), max(a, b)))
    bits = [1 if (i, j) in adj else 0 for j in range(1, n) for i in range(j)]
    bits += [0] * (-len(bits) % 6)
    body = bytes(63 + int("".join(map(str, bits[k:k + 6])), 2) for k in range(0, len(bits), 6))
    return _encode_size(n) + body


def read_graph6(source) -> Union[Graph, List[Graph]]:
    """Graphs from a graph6 file path, bytes or text: a list when there are
    several records, the graph itself when there is one (networkx's
    read_graph6 convention, which the reference relies on)."""
    if isinstance(source, (bytes, bytearray)):
        data = bytes(source)
    elif isinstance(source, str) and os.path.exists(source):
        with open(source, "rb") as f:
            data = f.read()
    elif isinstance(source, str):
        data = source.encode("ascii")
    else:
        data = source.read()
    graphs = [graph6_to_graph(line.strip()) for line in data.splitlines() if line.strip()]
    return graphs[0] if len(graphs) == 1 else graphs


def write_graph6(graphs: Iterable, path: str = None, header: bool = False) -> bytes:
    """graph6 text of ``graphs`` (one record per line); written to ``path``
    when given."""
    out = b"".join((b">>graph6<<" if header else b"") + graph_to_graph6(g) + b"\n" for g in graphs)
    if path is not None:
        with open(path, "wb") as f:
            f.write(out)
    return out


def load_stdgraphs(size: int, path: str = None) -> List[Graph]:
    """The 100-graph validation set for ``size`` nodes (6..32): read from
    ``path``/graph{size}er100.g6 when a directory is given, else a seeded
    synthetic set of 100 G(size, 0.5) graphs with the same shape."""
    if size < 6 or size > 32:
        raise ValueError("Size out of range.")
    if path is not None:
        graphs = read_graph6(os.path.join(path, f"graph{size}er100.g6"))
        return graphs if isinstance(graphs, list) else [graphs]
    return [gnp_random_graph(size, 0.5, seed=1000 * size + k) for k in range(100)]
