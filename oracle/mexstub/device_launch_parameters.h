/* empty: the oracle build needs no CUDA runtime declarations */
