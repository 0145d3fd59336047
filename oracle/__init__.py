"""Test infrastructure only: the CPU oracle for the CCT Biot-Savart / RK4 path.

Nothing in the product package imports this directory.  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline / reference arm use
it, and only as the checker or the timed CPU reference.
"""
