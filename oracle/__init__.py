"""FP64 CPU restatement of the reference's sphere mobility path (test infrastructure only)."""
