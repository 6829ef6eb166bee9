"""Data-driven callers of the ALS pattern (alternating ridge regression)."""
