"""FP64 CPU oracle of the GooFit fit path: test infrastructure only."""
