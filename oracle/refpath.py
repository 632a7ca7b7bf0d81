"""Where the reference's sources are read from (test infrastructure only).

The reference tree is read, never written, by the oracle recipes
(oracle/ref/Makefile), the plugin build tests and the fixture scripts.  Its
location comes from the QHG4_REF environment variable; the default is the
reference's checkout in the build container.  Machines without the tree
(the GPU hosts) skip what needs it.
"""
import os

REFERENCE_DIR = os.environ.get("QHG4_REF", "/root/reference/QHG4")


def reference_present() -> bool:
    return os.path.isdir(REFERENCE_DIR)
