"""Test infrastructure: the CPU oracle for libmobility_gb300 (see oracle.py)."""
