"""CPU oracle of the CVL primitive path (test infrastructure only)."""
