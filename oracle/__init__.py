"""Test oracle for the align-to-center path (checker only; see oracle.py)."""
