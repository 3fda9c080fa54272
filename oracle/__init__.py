"""CPU oracle for the HMC molecular-dynamics path (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` import this package, and only as the checker or the timed CPU
baseline -- never as part of the product path.
"""
