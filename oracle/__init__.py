"""CPU oracle of the MD step (test infrastructure only; see oracle.py)."""
