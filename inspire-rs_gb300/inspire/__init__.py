"""GB300-native InsPIRe server Respond path (drop-in for igor53627/inspire-rs).

The package mirrors the crate's Respond API (`inspire::pir`) over the C ABI of
include/inspire_gpu.h; all arithmetic runs in the CUDA kernels of csrc/.
"""
from .params import InspireParams, InspireVariant, num_columns  # noqa: F401
from .pir import (  # noqa: F401
    ClientPackingKeys,
    ClientQuery,
    EncodedDatabase,
    PinnedBuffer,
    PirError,
    RlweCiphertext,
    SeededClientQuery,
    Server,
    ServerCrs,
    ServerResponse,
    client_keygen_device,
    galois_keygen_device,
    external_product_device,
    now_ns,
    ntt_forward_device,
    ntt_inverse_device,
    query_seeded_device,
    respond,
    respond_batch,
    respond_inspiring,
    respond_one_packing,
    respond_seeded,
    respond_seeded_batch,
    respond_seeded_batch_device,
    respond_seeded_inspiring,
    respond_seeded_nopacking_batch,
    respond_seeded_packed,
    respond_seeded_packed_batch,
    respond_seeded_with_variant,
    respond_with_variant,
    write_crs_json,
    setup_keygen_device,
)
from . import wire  # noqa: F401,E402
