"""The oracle: CPU restatement of PixelFlow's OpenMP step (test infrastructure only)."""
