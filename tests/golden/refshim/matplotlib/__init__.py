"""No-op stand-in for ``matplotlib`` (the reference only plots progress).
Test infrastructure for fixture generation only."""
