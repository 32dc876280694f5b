"""FP64 CPU oracle (test infrastructure only; never imported by the engine)."""
