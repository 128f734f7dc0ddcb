"""GB300-native EBIV decode path for govid.

The decoder runs as hand-written sm_103a CUDA kernels behind the C-ABI in
``include/ebivgpu.h``; this package is the host-side mirror of govid's
``ebiv`` plugin API (Codec / Reader / Encoder) over that library.
"""
from . import ebiv  # noqa: F401
from .ebiv import (EOF, Codec, Config, EbivError, Encoder, ErrBadMagic, ErrConfig, ErrCorrupt,  # noqa: F401
                   ErrDimensions, ErrNoKeyframe, ErrUnsupported, ErrVersion, Frame, NewCodec, NewDemuxer,
                   Packet, Reader)

__all__ = ["ebiv", "Codec", "Reader", "Encoder", "Config", "Packet", "Frame", "NewCodec", "NewDemuxer",
           "EbivError", "ErrCorrupt", "ErrNoKeyframe", "ErrDimensions", "ErrUnsupported", "ErrVersion",
           "ErrBadMagic", "ErrConfig", "EOF"]
