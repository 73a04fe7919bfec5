"""ORACLE -- test infrastructure only, never part of the product.

CPU restatements of the reference's sparse-PCA path (brisc/pca.pyx,
brisc/cyutils.pyx, brisc/normalize.pyx, brisc/cysparse.pyx) and an FP64
ground truth. Imported only by tests/, __graft_entry__.smoke() and bench.py's
cpu_baseline leg, as the checker. The reference's own compiled modules, when
built by oracle/build_ref.py, live in oracle/_ref/ and are loaded by ref.py.
"""
