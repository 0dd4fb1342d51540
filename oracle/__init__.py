"""ORACLE — test infrastructure only (CPU restatement of SPECTER's hot path)."""
