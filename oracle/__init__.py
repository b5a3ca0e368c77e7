"""ORACLE TEST INFRASTRUCTURE — not part of the product: a plain-C restatement
of the reference's time-step loop and a harness over the reference's own
objects.  Only tests/, the smoke check and bench.py's CPU-baseline leg use it."""
