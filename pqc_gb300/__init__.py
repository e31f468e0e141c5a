"""pqcgpu: batched post-quantum KEMs on GB300 (sm_103a) behind the C ABI of include/pqcgpu.h."""
import os

# Independent batches run on many streams at once (mixed batches, the serving loop's slots).  The
# GPU multiplexes streams onto hardware work queues; with the default 8 queues a short kernel can
# wait behind another stream's queued kernel.  32 queues keep the streams apart.  Takes effect only
# if set before the process creates its CUDA context, so it is set on import.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
