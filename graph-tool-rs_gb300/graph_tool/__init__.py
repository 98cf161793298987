"""graph_tool (GB300 build): the centrality power iteration of graph-tool-rs
on one NVIDIA GB300, behind the reference's Python module surface.

    from graph_tool._rust import Graph
    g = Graph(); g.add_vertex(3); g.add_edge(0, 1); g.add_edge(1, 2)
    rank = g.new_vertex_property("double")
    sweeps = g.pagerank(rank)                 # centrality.rs:234-248

    from graph_tool.centrality import pagerank
    rank = pagerank(g)                        # graph-tool's signature

    g = load_graph("karate.gt")               # .gt reader, adjacency decoded on the GPU
"""
from ._rust import Graph, GraphBatch, PropertyMap, value_types  # noqa: F401
from .gt import GtFile, load_graph  # noqa: F401

__all__ = ["Graph", "GraphBatch", "PropertyMap", "value_types", "GtFile", "load_graph"]
