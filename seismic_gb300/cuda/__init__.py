"""Drop-in for the reference's CUDA wrapper module (see correlation_lib)."""
