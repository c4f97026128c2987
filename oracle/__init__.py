"""CPU parity oracle for the OSIRIS PIC time step -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may import
this package.  The product (``osiris_gb300``) never does.
"""
