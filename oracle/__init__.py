"""CPU oracle for the parity tests (test infrastructure only; see oracle.py)."""
