"""CPU oracle (test infrastructure only): a restatement of the reference
server algorithm used as the checker for the CUDA path."""
