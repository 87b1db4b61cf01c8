"""Oracle: FP64 CPU restatement of ma-shm's flat-shell loop (test infrastructure only)."""
