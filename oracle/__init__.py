"""CPU oracle for the NSST hot path: TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import anything here, as the checker or as the timed CPU
baseline.  The product (``shearcuda_gb300``) never imports it."""
