"""CPU oracle for the PathFinder hot path (test infrastructure only).

This package restates, on the CPU, the algorithms of OrthoRoute's PathFinder
negotiated-congestion loop that the GB300 build accelerates.  It exists to
check the CUDA path: only the test suite, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` leg of ``bench.py`` may import it.  The product package
(``orthoroute_gb300``) never imports, links or executes anything from here.

Parity is pinned: ``tests/golden/make_golden.py`` drives the reference's own
functions on seeded inputs and the committed fixtures under ``tests/golden/``
are compared against these restatements by ``tests/test_oracle_golden.py``.

Modules
-------
lattice     A1  lattice → CSR graph (edge order identical to the reference)
accounting  A2–A5  cost update, live present, history, via pools
roi         A6  bidirectional BFS region of interest
dijkstra    A7–A8  heap Dijkstra with FP64 labels / FP32 distances, backtrace
tallies     A8–A9  path → arcs, overuse, node use, barrel conflicts
"""
