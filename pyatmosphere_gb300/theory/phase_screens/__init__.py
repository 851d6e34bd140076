"""Phase-screen theory helpers (the reference's theory/phase_screens package)."""
