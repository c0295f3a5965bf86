"""The reference's own code compiled here (test infrastructure): see
build_ref.py for the recipe and reference.py for the ctypes binding."""
