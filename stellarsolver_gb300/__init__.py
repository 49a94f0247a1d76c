"""GB300 (sm_103a) 2D Barnes-Hut engine with the surface of pentilm/StellarSolver.

The compute path is the C-ABI library lib/libstellar_bh.so (include/stellar_bh.h);
this package is its Python binding (`bh`), the in-tree build (`build`) and the
initial-condition models (`models`).  There is no CPU fallback: importing `bh`
on a machine without the built library raises.
"""
__version__ = "0.1.0"
