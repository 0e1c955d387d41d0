"""Oracle package: CPU restatement of the tbslas SL path (test infrastructure only)."""
