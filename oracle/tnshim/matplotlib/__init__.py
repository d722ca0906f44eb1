"""Import stub for matplotlib (absent here).  Any use raises."""
