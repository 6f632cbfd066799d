"""ORACLE -- test infrastructure only (the checker of tests/, smoke() and the
cpu_baseline leg of bench.py); the product never imports it."""
