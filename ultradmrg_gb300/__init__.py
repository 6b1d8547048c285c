"""GB300-native two-site DMRG/TDVP local update (block-sparse matvec, Lanczos,
environment update, truncated block SVD) behind a C ABI."""
