"""graph-tool's functional centrality interface over the GPU solves.

``pagerank``, ``eigenvector`` and ``betweenness`` take graph-tool's keyword arguments
(``graph_tool.centrality.pagerank(g, damping, pers, weight, prop, epsilon,
max_iter, ret_iter)``) and call the same kernels as ``Graph.pagerank`` /
``Graph.eigenvector``: crates/gt-algo/src/centrality.rs:234-384 and :405-497
of graph-tool-rs.  ``max_iter=None`` means no cap (centrality.rs:84-88).
"""
from __future__ import annotations

from ._rust import Graph, PropertyMap


def pagerank(g: Graph, damping: float = 0.85, pers: PropertyMap | None = None,
             weight: PropertyMap | None = None, prop: PropertyMap | None = None,
             epsilon: float = 1e-6, max_iter: int | None = None, ret_iter: bool = False,
             grain: int = 4096, precision: str = "f32"):
    """PageRank of every vertex; ``prop`` (if given) is the initial iterate
    and receives the result."""
    rank = prop if prop is not None else g.new_vertex_property("double")
    it = g.pagerank(rank, weight=weight, pers=pers, damping=damping, epsilon=epsilon,
                    max_iter=max_iter or 0, grain=grain, precision=precision)
    return (rank, it) if ret_iter else rank


def eigenvector(g: Graph, weight: PropertyMap | None = None, vprop: PropertyMap | None = None,
                epsilon: float = 1e-6, max_iter: int | None = None, grain: int = 4096,
                precision: str = "f32"):
    """(eigenvalue, centrality map), as graph-tool returns them."""
    x = vprop if vprop is not None else g.new_vertex_property("double")
    eig, _ = g.eigenvector(x, weight=weight, epsilon=epsilon, max_iter=max_iter or 0,
                           grain=grain, precision=precision)
    return eig, x


def betweenness(g: Graph, vprop: PropertyMap | None = None, eprop: PropertyMap | None = None,
                undirected: bool = False):
    """(vertex betweenness, edge betweenness), unnormalised, every vertex a
    pivot (crates/gt-algo/src/centrality.rs:633-689)."""
    return g.betweenness(vprop, eprop, undirected=undirected)
