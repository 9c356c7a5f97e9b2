"""f2py-compatible replacement of the reference's misc.f_misc module."""
