"""diffren_gb300 (package init placeholder)."""
