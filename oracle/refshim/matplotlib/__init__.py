"""Empty ``matplotlib`` stand-in for the oracle harness (no plotting here)."""
