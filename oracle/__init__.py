"""CPU oracle of the WCSPH step (test infrastructure; see oracle/binding.py)."""
