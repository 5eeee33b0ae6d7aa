"""Oracle build helper (test infrastructure only): where the reference checkout is.

The reference's sources are read in place, never copied: the GLSL harness
(``oracle/glsl_cpu``) compiles them and the fixture scripts under
``tests/golden/`` import its host Python. Their location is the
``FLOWX_REFERENCE`` environment variable, read at every call; when it is unset
the recipes look at the build container's mount point. Machines without the
checkout (the GPU host) never need it: they use the committed fixtures.
"""

from __future__ import annotations

import os

ENV = "FLOWX_REFERENCE"
MOUNT = "/root/reference"


def checkout() -> str:
    """The reference checkout's root directory."""
    return os.environ.get(ENV) or MOUNT


def available() -> bool:
    """Whether the checkout (its shader sources) is present here."""
    return os.path.isdir(os.path.join(checkout(), "shaders"))
