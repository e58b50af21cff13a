"""TEST INFRASTRUCTURE ONLY: CPU oracle for parity tests (see oracle.py)."""
