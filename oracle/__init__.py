"""Test infrastructure: CPU oracles of the geodesic render (see oracle.py,
refbridge.py, build_ref.py). Imported only by the tests, the smoke check and
the CPU-baseline leg of the bench."""
