"""No-op stand-in for matplotlib, put on PYTHONPATH only for the reference
wrapper test (matplotlib is not installed; the wrapper only plots with it)."""
