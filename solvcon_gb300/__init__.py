"""solvcon-gb300: solvcon's CESE time-march re-built for the NVIDIA GB300.

The public surface mirrors the reference's Python classes for this path:
``StaticMesh``, ``EulerCore``, ``GradientElement``, ``EulerField``,
``Euler1DCore``/``Euler1DSolver``/``ShockTube`` and the spacetime scalar
solvers.  All march arithmetic runs in hand-written sm_103a CUDA kernels in
the native library ``_lib/libscg.so``; importing the package without that
library raises ImportError.
"""

from .buffer import SimpleArray  # noqa: F401
from .mesh import Gmsh, Plot3d, StaticMesh, StaticMeshBc  # noqa: F401
from .multidim import EulerCore, GradientElement  # noqa: F401
from .host import HostTable  # noqa: F401
from .field import EulerField  # noqa: F401

__version__ = "0.1.0"
