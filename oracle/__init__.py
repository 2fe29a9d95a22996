"""Oracle: CPU restatement of the reference's sampled-ALS path (test infrastructure only)."""
