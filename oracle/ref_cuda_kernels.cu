/*
 * TEST INFRASTRUCTURE ONLY.  The reference's own CUDA kernels for the BAM
 * path, compiled from their sources where they lie
 * (crates/fritillaria-cuda/kernels/inflate.cu and bam_decode.cu, reached
 * through -I) into one sm_103a cubin by oracle/build.py.  The kernels keep
 * their extern "C" names (inflate_blocks, bam_scan_blocks, bam_reconcile,
 * bam_emit_offsets, bam_decode_fields); each source sits in its own namespace
 * so their file-local helpers do not collide.  Nothing here is shipped; the
 * driver in ref_cuda_driver.cpp loads the cubin to time the reference's CUDA
 * path beside this library's.
 */
namespace ref_inflate {
#include "inflate.cu"
}
namespace ref_bam {
#include "bam_decode.cu"
}
