"""CPU oracle of the BEM hot path -- test infrastructure only (see port.py)."""
