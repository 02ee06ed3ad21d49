"""nebc7_gb300: BC7 block encoder for NVIDIA GB300 (sm_103a).

Bit-exact to the andrewevstyukhin/nebc7 CPU encoder's per-block path (modes
0-7 and Mode6Index2, error stepping, per-channel weights, masks, incremental
re-encode).  The compute runs in hand-written CUDA kernels behind the C ABI
of include/nebc7_gb300.h; this package builds that library in-tree and wraps
it.
"""

from . import synth  # noqa: F401
from ._native import build, load, NativeError  # noqa: F401
from .api import (  # noqa: F401
    Bc7Core, Preset, DEFAULT, PRECISE, EncodeStats, EncodedImage,
    encode_image, encode_device, set_pca, pad_texture, outline_mask, padded_size, parse_flags, Batch, BatchTexture, PlanStore, plan_key, Server,
    ktx_header, write_ktx, read_ktx,
)
