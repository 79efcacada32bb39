// segsort.cuh -- device-wide exclusive scan and stable LSD radix sort
// (segsort.cu) for buffers sized by a host-known capacity whose live count
// sits in device memory.
#pragma once

#include "common.cuh"

namespace sg {

// ints of scratch an exclusive scan of n elements needs
size_t scan_scratch_ints(long n);

// Exclusive scan of in[0, n) into out (in place allowed); the sum into
// *total (may be null).  scratch: scan_scratch_ints(n) ints.
void launch_excl_scan(const int *in, long n, int *out, int *scratch, int *total, sg_stream_t stream);

// The same over the first min(*n_dev, n) elements (n_dev in device memory).
void launch_excl_scan_dev(const int *in, long n, const int *n_dev, int *out, int *scratch, int *total,
                          sg_stream_t stream);

// bytes of scratch a radix sort of up to cap items needs
size_t radix_scratch_bytes(long cap);

// Stable sort of (keys_in[i], vals_in[i]) for i < *n_dev (n_dev <= cap;
// vals_in null: the values are i) by the low key_bits bits of the keys, 8
// bits a pass; passes alternate between the (keys_a, vals_a) and (keys_b,
// vals_b) buffers, starting with a (the input may be the b pair).  Returns
// the number of passes: the result is in a when it is odd, in b when even.
int launch_radix_sort(const uint32_t *keys_in, const uint32_t *vals_in, const int *n_dev, long cap, int key_bits,
                      uint32_t *keys_a, uint32_t *vals_a, uint32_t *keys_b, uint32_t *vals_b, void *scratch,
                      sg_stream_t stream);

}  // namespace sg
