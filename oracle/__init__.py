"""Parity oracle: CPU FP64 restatement of EbbCFD's explicit FV update.

TEST INFRASTRUCTURE ONLY.  Imported by tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py``; the product package never imports it.
"""
