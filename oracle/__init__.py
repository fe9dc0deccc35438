"""CPU FP64 oracle of the elastic operator path: test infrastructure only (the parity reference)."""
