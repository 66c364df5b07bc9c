"""CPU oracle for the particular acceleration hot path (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py`` may import
this package. The product (``particular_gb300``) never imports it.
"""
