"""CPU FP64 oracle of the trace-and-accumulate path (test infrastructure only)."""
