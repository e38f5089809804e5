"""CPU oracle for the NSST hot path: TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` (its ``cpu_baseline`` and ``--impl reference``) may import
anything here, to check the GPU results against or as the timed CPU
baseline.  The product (``shearcuda_gb300``) never imports it."""
