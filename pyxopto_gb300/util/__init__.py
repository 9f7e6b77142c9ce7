"""Post-processing helpers (xopto/util)."""
