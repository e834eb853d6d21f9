"""Oracle package: test infrastructure only (CPU restatement of the reference; never shipped)."""
