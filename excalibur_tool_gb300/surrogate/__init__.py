"""Learned sky-map surrogate: BF16 tensor-core MLP ensemble trained on traced rays."""
