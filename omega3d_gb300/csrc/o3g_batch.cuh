// o3g_batch.cuh -- host-side interface of the batched persistent pair sums (o3g_batch.cu),
// shared with the batched Ralston stepper (o3g_rk2.cu).
#pragma once

#include "o3g_batch_impl.cuh"

namespace o3g {

// Creates a batch over nsys systems.  `binds` holds nbind host arrays of nsys descriptors
// (pointers and counts; the offsets are filled in here); every binding has the same counts
// and is run with the same plan (batch_run picks one).
int32_t batch_create(int core, int prec, bool grads, int nsys, const BatchSysDev* const* binds, int nbind,
                     o3g_batch_t** out);
// Queues the pair sums of binding `bind` on `st` (tunes first when the shape has no cached
// configuration and `st` is not capturing).
int32_t batch_run(o3g_batch_t* h, int bind, cudaStream_t st);
// Tunes now on binding 0 unless the shape is tuned already (force = retune anyway).
int32_t batch_tune(o3g_batch_t* h, cudaStream_t st, bool force);

}  // namespace o3g
