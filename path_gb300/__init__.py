"""GB300-native render hot path of the rgreenblatt/path tracer."""

from . import api, capi, scenes  # noqa: F401
from .api import (ExecutionModel, Renderer, RendererFromFiles, Scene, Settings,  # noqa: F401
                  SquareImage, camera_transform, material)
