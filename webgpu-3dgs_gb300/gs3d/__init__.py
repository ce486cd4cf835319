"""gs3d - GB300 (sm_103a) Gaussian-splat rebin path with the reference
renderer's host interface (see renderer.GaussianSplatRenderer)."""
from ._lib import BUFFERS, Gs3dError, LIB_PATH, load  # noqa: F401
from .camera import Camera, camera_struct  # noqa: F401
from .renderer import (PROJ_DTYPE, GaussianSplatRenderer, RenderFrameInfo, Scene,  # noqa: F401
                       SceneSyncer)
from .scenes import GaussianSplatData  # noqa: F401
from . import scenes  # noqa: F401
