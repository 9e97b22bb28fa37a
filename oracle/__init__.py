"""ORACLE — test infrastructure, not part of the product.

CPU restatement of the reference's render path (torch_port) and of the library's counter
hash (hash). Imported only by tests/, __graft_entry__.smoke() and bench.py's baseline
legs, always as the checker or the timed baseline, never by plenoxels_gb300.
"""
