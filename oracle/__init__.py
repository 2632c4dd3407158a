"""CPU oracle for wrach's per-frame particle physics step.

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and bench.py's
CPU-baseline leg, never by the product package.
"""
