/*
 * bpl_gb300.h -- C ABI of the GB300-native BP-Layers hot path.
 *
 * Every entry point takes caller-owned device pointers, plain sizes and a
 * CUDA stream (passed as void*; NULL = legacy default stream), enqueues its
 * kernels on that stream and returns a status code.  Nothing here
 * synchronises the device, exits the process or allocates device memory
 * unless stated.  All tensors are dense, contiguous, row-major float32 unless
 * stated, with the reference's layouts:
 *
 *   cost      (B,H,W,L)        messages / argmin  (B,4,H,W,L)
 *   edge      (Be,4,H,W)       scale              (B,4,H,W)
 *   stereo jump taps  (Bj,4,Lv,H,W)  [offset, ..., 0 at Lv/2, ...]
 *   semantic global   (1,4,L,L)      jump[d][s][t] = cost of label t given s
 *   semantic pixel    (4,H,W,L,L)
 *   direction index:  LEFT=0, RIGHT=1, UP=2, DOWN=3; message slot k at a
 *   pixel holds the message received from the neighbour on side k.
 *
 * Differences from the reference ops (deliberate, documented):
 *   - every batch item is processed (the reference forward/SAD/flow kernels
 *     only process batch item 0);
 *   - argmin may be stored as float32 (reference layout), uint8 or uint16.
 */
#ifndef BPL_GB300_H
#define BPL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define BPL_OK 0
#define BPL_ERR_INVALID_ARG 1
#define BPL_ERR_UNSUPPORTED 2
#define BPL_ERR_CUDA 3
#define BPL_ERR_DEVICE_TIMEOUT 4

/* LBP pairwise variants */
#define BPL_LBP_STEREO 0      /* ops/lbp_stereo            */
#define BPL_LBP_SEM_GLOBAL 1  /* ops/lbp_semantic_pw       */
#define BPL_LBP_SEM_PIXEL 2   /* ops/lbp_semantic_pw_pixel */
/* ops/lbp_semantic_pw_pixel with the layer's input instead of the op's: the
 * pairwise tensor is (2,H,W,L,L) (LR and UD planes) and the kernels apply the
 * shift and transpose that LBPMinSumFunction.forward materialises as
 * (4,H,W,L,L) (message_passing_op_pw_pixel.py:27-38); grad_jump is
 * (2,H,W,L,L), the fold of its backward (:47-51). */
#define BPL_LBP_SEM_PIXEL_LAYER 3

/* argmin storage */
#define BPL_ARGMIN_NONE 0
#define BPL_ARGMIN_F32 1
#define BPL_ARGMIN_U8 2
#define BPL_ARGMIN_U16 3

/* library version (major*10000 + minor*100 + patch) */
int bpl_version(void);

/* static text for a status code */
const char* bpl_status_string(int status);

/* message describing the last failure of a call made on this host thread */
const char* bpl_last_error(void);

/* Reads and clears the device error word that kernels set when one of their
 * bounded waits runs out (synchronises the current device).  *code receives 0
 * when no kernel reported an error. */
int bpl_read_device_error(int* code);

/* Sets the number of polls after which the kernels' bounded waits (the
 * mbarrier waits of the TMA-staged pixel-pairwise LBP forward and of the flow
 * SAD forward) give up, raise the device error word and return early with
 * their outputs incomplete.  BPL_DEFAULT_WAIT_LIMIT (the value at load) is
 * far beyond any copy's latency.  For tests of the timeout path: 0 makes
 * every wait give up at once while the copies it waits for still land (a
 * kernel whose wait gave up waits for its copies in flight before it exits).
 * Applies to the current device.  No counterpart in the reference, whose
 * kernels have no waits. */
#define BPL_DEFAULT_WAIT_LIMIT 16777216u
int bpl_set_wait_limit(unsigned polls);

/*
 * Min-sum LBP forward: one pass of the four directional sweeps (RIGHT, LEFT,
 * DOWN, UP), messages updated in place.
 * Replaces cuda::lbp_forward_min_sum / lbp_reduction_min_sum
 *   ops/lbp_stereo/src/lbp_min_sum_kernel.cu:424-508   (variant STEREO)
 *   ops/lbp_semantic_pw/src/lbp_min_sum_kernel.cu:424-510   (SEM_GLOBAL)
 *   ops/lbp_semantic_pw_pixel/src/lbp_min_sum_kernel.cu:421-506 (SEM_PIXEL)
 * bound in Python as `forward_minsum` (ops/lbp_stereo/src/lbp.cpp:16-27, :53).
 *
 * jump_batch / edge_batch: leading extent of jump (stereo only) and edge,
 * 1 (broadcast) or B.  Lv: number of stereo jump taps (2..16; ignored for the
 * semantic variants).  delta: truncation half-width (the reference's uint16
 * `delta`; delta >= L selects the full O(L^2) minimisation).  argmin: output
 * of `argmin_kind` type laid out like messages, or NULL with
 * BPL_ARGMIN_NONE.  scale: (B,4,H,W) per-message exp-sum.  Only the
 * receiving positions of each sweep are written (as in the reference); the
 * caller zero-fills argmin/scale if it needs the rest defined.
 * L: 1..1024.  Results are bit-identical to the reference's arithmetic.
 */
int bpl_lbp_forward(int variant, const float* cost, const float* jump, const float* edge,
                    float* messages, void* argmin, int argmin_kind, float* scale, int B, int H,
                    int W, int L, int Lv, int jump_batch, int edge_batch, int delta, void* stream);

/*
 * LBP forward with FP16 storage: cost and messages (and the pixel-pairwise
 * matrices) stored as IEEE half, all arithmetic in FP32, the normalisation's
 * exp by the hardware approximation.  No counterpart in the reference
 * (which is FP32 only); same sweeps and tie rules as bpl_lbp_forward.
 * Stored messages are referenced to the minimum of h instead of
 * log-normalised: row = m_raw - min_s h(s), scale = sum_t exp(row[t]), so
 * the reference's normalised message is row - log(scale).  Beliefs built
 * from them differ from the reference's by a constant per pixel (their
 * argmin and softmin are unchanged), and half's finest steps fall on the
 * labels near the row's minimum.
 * Layout: the label axis has stride Lp = L rounded up to 8 (16-byte rows):
 *   cost (B,H,W,Lp) half, messages (B,4,H,W,Lp) half, argmin (B,4,H,W,Lp),
 *   pixel-pairwise jump (4,H,W,L,Lp) half; stereo jump taps, the semantic
 *   global jump (1,4,L,L), edge and scale stay float.  Labels L..Lp-1 are
 *   ignored on input and not written.
 * scale may be NULL: it is then not computed (the FP16 adjoint recomputes
 * the normalisation from the rows), and the stereo kernel's step carries no
 * exp at all.
 * Variants: all (BPL_LBP_STEREO, BPL_LBP_SEM_GLOBAL, BPL_LBP_SEM_PIXEL[_LAYER]).
 */
int bpl_lbp_forward_f16(int variant, const void* cost, const void* jump, const float* edge,
                        void* messages, void* argmin, int argmin_kind, float* scale, int B, int H,
                        int W, int L, int Lv, int jump_batch, int edge_batch, int delta, void* stream);

/* Bytes of device workspace bpl_lbp_backward needs: B*2*H*W*L floats (the
 * vertical sweeps' chain gradients that the horizontal sweeps read; the
 * reference allocates the same as saved_prev_grad_msg,
 * ops/lbp_stereo/src/lbp_min_sum_kernel.cu:538). */
size_t bpl_lbp_backward_workspace_size(int B, int H, int W, int L);

/*
 * Reference adjoint of one LBP pass ("backward_minsum").
 * Replaces cuda::lbp_backward_min_sum
 *   ops/lbp_stereo/src/lbp_min_sum_kernel.cu:513-621          (STEREO)
 *   ops/lbp_semantic_pw/src/lbp_min_sum_kernel.cu:516-624      (SEM_GLOBAL)
 *   ops/lbp_semantic_pw_pixel/src/lbp_min_sum_kernel.cu:512-620 (SEM_PIXEL)
 * bound in Python as `backward_minsum` (ops/lbp_stereo/src/lbp.cpp:29-46).
 *
 * Inputs: in_grad (B,4,H,W,L) upstream gradient of the messages; messages,
 * argmin (argmin_kind F32/U8/U16) and scale as returned by bpl_lbp_forward.
 * Outputs (zero-filled by this call, then accumulated):
 *   grad_cost (B,H,W,L);
 *   grad_jump: STEREO (jump_batch,4,Lv,H,W); SEM_GLOBAL (B,4,L,L) with the
 *     gradient of the shared matrix summed into batch item 0, like the
 *     reference; SEM_PIXEL (4,H,W,L,L);
 *   grad_edge (edge_batch,4,H,W) (NULL allowed for SEM_PIXEL, which has no
 *     edge gradient in the reference).
 * The message gradient of the reference op is in_grad itself (the caller
 * copies it if it needs a distinct tensor).  jump may be NULL for SEM_PIXEL.
 * workspace: device scratch of bpl_lbp_backward_workspace_size() bytes.
 * Float atomics make the summation order, and so the last bits, vary from
 * run to run, as in the reference.
 */
int bpl_lbp_backward(int variant, const float* jump, const float* edge, const float* in_grad,
                     const float* messages, const void* argmin, int argmin_kind, const float* scale,
                     float* grad_cost, float* grad_jump, float* grad_edge, void* workspace,
                     size_t workspace_bytes, int B, int H, int W, int L, int Lv, int jump_batch,
                     int edge_batch, void* stream);

/*
 * Reference adjoint of `passes` LBP passes run in place on one messages
 * tensor (the reference's iteration loop, message_passing_op_cuda.py:161-168):
 * its backward of every pass reads the same messages (the last pass's, the
 * tensor having been overwritten) and the same in_grad (the message gradient
 * it returns is in_grad), so the passes' adjoints are independent and run
 * here as one launch.  argmin (passes,B,4,H,W,L) and scale (passes,B,4,H,W)
 * are stacked in pass order; grad_cost, grad_jump and grad_edge receive the
 * sum over the passes (what the reference's autograd accumulates).
 * in_grad is read with the given strides in elements between batch items
 * and between message slots (4*H*W*L and H*W*L for a (B,4,H,W,L) tensor;
 * slot stride 0 reads one (B,H,W,L) gradient for all four slots, which is
 * what the beliefs' sum over the slots produces).
 * workspace: passes * bpl_lbp_backward_workspace_size(B, H, W, L) bytes.
 * No counterpart in the reference (one call per pass there); other
 * arguments as bpl_lbp_backward.
 */
int bpl_lbp_backward_passes(int variant, const float* jump, const float* edge, const float* in_grad,
                            int64_t in_grad_batch_stride, int64_t in_grad_slot_stride,
                            const float* messages, const void* argmin, int argmin_kind, const float* scale,
                            float* grad_cost, float* grad_jump, float* grad_edge, void* workspace,
                            size_t workspace_bytes, int B, int H, int W, int L, int Lv, int jump_batch,
                            int edge_batch, int passes, void* stream);

/* The same for FP16 storage (layout of bpl_lbp_backward_f16; workspace
 * passes * bpl_lbp_backward_workspace_size(B, H, W, Lp) bytes). */
int bpl_lbp_backward_passes_f16(int variant, const float* jump, const float* edge, const void* in_grad,
                                int64_t in_grad_batch_stride, int64_t in_grad_slot_stride,
                                const void* messages, const void* argmin, int argmin_kind, const float* scale,
                                float* grad_cost, float* grad_jump, float* grad_edge, void* workspace,
                                size_t workspace_bytes, int B, int H, int W, int L, int Lv, int jump_batch,
                                int edge_batch, int passes, void* stream);

/*
 * bpl_lbp_backward_passes (storage 0, float messages) or
 * bpl_lbp_backward_passes_f16 (storage 1) with the cost gradient added onto
 * what grad_cost holds instead of written: each contribution times
 * cost_sign (+1 or -1), label stride grad_cost_ls (L, or Lp = L rounded up
 * to 8 for half storage).  grad_cost is not zeroed and must not alias
 * in_grad.  The layer's fused backward passes the buffer holding the
 * gradient of the probability volume (cost = -prob) from the belief
 * epilogue, with cost_sign -1, so the sum and the negation of the two cost
 * gradients cost no extra pass.  layer_taps = 1 (stereo, Lv = 6): jump is
 * the layer's packed taps [offset, L2, L1-, 0, L1+, L2] (taps 1 and 5 equal,
 * tap 3 zero), and grad_jump receives what the layer's fold needs: the two
 * L2 taps' gradient summed in tap 1, none in taps 3 and 5
 * (message_passing_op_cuda.py:75-93 adds taps 1 and 5 and drops tap 3).
 * No counterpart in the reference (autograd adds the cost's gradients
 * there).
 */
int bpl_lbp_backward_passes_into(int storage, int variant, const float* jump, const float* edge, const void* in_grad,
                                 int64_t in_grad_batch_stride, int64_t in_grad_slot_stride, const void* messages,
                                 const void* argmin, int argmin_kind, const float* scale, float* grad_cost,
                                 int grad_cost_ls, float cost_sign, float* grad_jump, float* grad_edge,
                                 void* workspace, size_t workspace_bytes, int B, int H, int W, int L, int Lv,
                                 int jump_batch, int edge_batch, int passes, int layer_taps, void* stream);

/*
 * Exact adjoint of one LBP pass (FP32 storage).  No counterpart in the
 * reference, whose adjoint (bpl_lbp_backward) returns in_grad as the message
 * gradient; the cost, jump and edge gradients are the reference adjoint's
 * (the reference carries the vertical sweeps' accumulators without the
 * normalisation's Jacobian, which is exact because every vector that
 * Jacobian's transpose produces sums to zero).  grad_messages (B,4,H,W,L)
 * receives the gradient with respect to the pass's input messages: the
 * vertical messages read by the horizontal sweeps at every pixel, the chain
 * inputs at each sweep's first sender, and, for the slots the pass never
 * writes (LEFT at x=0, RIGHT at x=W-1, UP at y=0, DOWN at y=H-1), the
 * upstream gradient passing through plus the vertical sweeps' reads.  With
 * it the gradient of several chained passes is the derivative of the
 * forward (checked against central finite differences in FP64 on the
 * oracle).  Other arguments as bpl_lbp_backward.
 */
int bpl_lbp_backward_exact(int variant, const float* jump, const float* edge, const float* in_grad,
                           const float* messages, const void* argmin, int argmin_kind, const float* scale,
                           float* grad_cost, float* grad_jump, float* grad_edge, float* grad_messages,
                           void* workspace, size_t workspace_bytes, int B, int H, int W, int L, int Lv,
                           int jump_batch, int edge_batch, void* stream);

/*
 * Fused belief epilogue (no counterpart in the reference, which runs
 * messages.sum(dim=1) + cost and TemperatureSoftmin as separate torch
 * passes: ops/lbp_stereo/message_passing_op_cuda.py:170-173,
 * corenet.py:106-113).  beliefs (B,H,W,L) = softmin(z / T) over labels with
 * z = (((M0 + M1) + M2) + M3) + cost; messages (B,4,H,W,Ls) float
 * (messages_half = 0) or half (1, Ls = L rounded up to 8), cost (B,H,W,L);
 * temperature: one device float (read on the device, so no host sync).
 */
int bpl_beliefs_forward(const void* messages, int messages_half, const float* cost, const float* temperature,
                        float* beliefs, int B, int H, int W, int L, int Ls, void* stream);

/*
 * Its backward: grad_z (B,H,W,L) = d loss / d z (also each message slot's
 * gradient) from beliefs and grad_beliefs; grad_temperature (one device
 * float, zeroed by this call, may be NULL) = d loss / d T, for which z is
 * recomputed from messages and cost.
 */
int bpl_beliefs_backward(const void* messages, int messages_half, const float* cost, const float* temperature,
                         const float* beliefs, const float* grad_beliefs, float* grad_z, float* grad_temperature,
                         int B, int H, int W, int L, int Ls, void* stream);

/*
 * bpl_beliefs_forward with z = sum + cost_sign * cost (cost_sign +1 or -1:
 * -1 reads the layer's probability volume, whose negation the cost is) and
 * the cost in either storage: cost_half = 0, (B,H,W,L) float; 1, the
 * FP16-storage volume (B,H,W,Ls) half (Ls = L rounded up to 8).  log_norm
 * (B,H,W) float, may be NULL: per pixel c = min(z/T) - log(sum of the
 * softmin's exps), from which bpl_beliefs_backward_ex recovers z/T as
 * c - log(beliefs).
 */
int bpl_beliefs_forward_ex(const void* messages, int messages_half, const void* cost, int cost_half,
                           float cost_sign, const float* temperature, float* beliefs, float* log_norm, int B, int H,
                           int W, int L, int Ls, void* stream);

/*
 * bpl_beliefs_backward for the layer's fused backward: cost and cost_sign as
 * bpl_beliefs_forward_ex; grad_z (B,H,W,L) receives
 * grad_z_sign (+1 or -1) times d loss / d z, and grad_copy, by copy_kind, a
 * second copy of +d loss / d z: 0 none, 1 (B,H,W,Ls) half with the padding
 * zeroed (the FP16 adjoint's in_grad), 2 (B,4,H,W,L) float in every message
 * slot (the message gradient of a leaf message tensor), 3 (B,H,W,L) float.
 * log_norm: the forward's, or NULL to recompute z from messages and cost for
 * grad_temperature (with it, messages and cost are not read and may be
 * NULL).
 */
int bpl_beliefs_backward_ex(const void* messages, int messages_half, const void* cost, int cost_half,
                            float cost_sign, const float* temperature, const float* beliefs, const float* grad_beliefs, float* grad_z,
                            float grad_z_sign, void* grad_copy, int copy_kind, float* grad_temperature,
                            const float* log_norm, int B, int H, int W, int L, int Ls, void* stream);

/*
 * dst (B,4,n) = src (B,n) repeated over the four message slots; elements of
 * elem_bytes (4: float, 2: half).  The message gradient of the reference's
 * backward (grad_messages = in_grad, ops/lbp_stereo/src/lbp_min_sum_kernel.cu:
 * 534-536) when in_grad is the beliefs' gradient broadcast over the slots,
 * written out for a leaf message tensor.
 */
int bpl_broadcast_slots(const void* src, void* dst, int B, int64_t row_elems, int elem_bytes, void* stream);

/*
 * Coarse-to-fine glue (stereo.py:104-113): pv (N,2h,2w,2d) += weight *
 * trilinear x2 upsampling of beliefs (N,h,w,d) over rows, columns and labels
 * (F.interpolate(scale_factor=2.0, mode='trilinear'), align_corners False;
 * the reference adds it halved: weight 0.5).  In place on pv, one pass.
 */
int bpl_upsample_add_beliefs(const float* beliefs, float* pv, int N, int h, int w, int d, float weight,
                             void* stream);

/*
 * Cost volume from a SAD volume (the reference's matching step,
 * matching.py:22-25, followed by MessagePassing's cost = -prob,
 * message_passing_op_cuda.py:162): cost[n,y,x,t] = -softmax_t(-sad[n,y,x,t] /
 * temperature) over the D disparities, in one pass.  sad (B,H,W,D) float;
 * cost (B,H,W,Ls) float (cost_half = 0) or half (1), labels D..Ls-1 of each
 * row set to zero (Ls = D, or D rounded up to 8 for the FP16-storage
 * layout).  exp by expf and the sum in any order: within float rounding of
 * torch's softmax, not bit-identical to it.  No counterpart in the
 * reference's ops (torch calls there).
 */
int bpl_cost_from_sad(const float* sad, void* cost, int cost_half, int B, int H, int W, int D, int Ls,
                      float temperature, void* stream);

/*
 * Per-pixel disparity straight from the messages: disparity[n,y,x] =
 * argmin_t ((((M0 + M1) + M2) + M3) + cost)[t], first index on ties: the
 * label whose belief softmin(...) is largest (the reference's
 * MessagePassing beliefs followed by Inference "wta",
 * message_passing_op_cuda.py:170-173, inference_op.py:23-27), without the
 * belief volume.  messages (B,4,H,W,Ls) float or half (messages_half); cost
 * (B,H,W,Lc) float or half (cost_half); disparity (B,H,W) int32 or int64
 * (disparity_int64).  No counterpart in the reference.
 */
int bpl_messages_argmin(const void* messages, int messages_half, const void* cost, int cost_half,
                        void* disparity, int disparity_int64, int B, int H, int W, int L, int Ls, int Lc,
                        void* stream);

/*
 * Inference on a belief volume (B,H,W,L) float (Inference.forward,
 * ops/lbp_stereo/inference_op.py:22-97): mode 0 "wta", out (B,H,W) int64 =
 * argmax over labels (first index, as torch.argmax); mode 1 "sub-exp", out
 * (B,H,W) float = the expectation of the label over the argmax's
 * +-support window, window labels clamped to [0, L-1], renormalised
 * (compute_sub_expectation, :53-97; support <= 15).  One pass instead of
 * the reference's gather and three reductions.
 */
int bpl_beliefs_infer(const float* beliefs, int mode, int support, void* out, int B, int H, int W, int L,
                      void* stream);

/*
 * Stereo jump taps from per-pixel affinities, in one pass
 * (LBPMinSumFunction.forward, ops/lbp_stereo/message_passing_op_cuda.py:35-60):
 * affinities (N,4,K,H,W) [L2-, L2+, L1-, L1+, L3] (K = 5) or [L1, L1, L2]
 * (K = 3) and offset (N,4,H,W) -> taps (N,4,K+3,H,W)
 * [offset, L3, .., 0, .., L3], the pairs of directions RIGHT-to-LEFT and
 * DOWN-to-UP in reverse order.  K odd, 3..13.
 */
int bpl_pack_taps(const float* affinities, const float* offset, float* taps, int N, int K, int H, int W,
                  void* stream);

/*
 * Its gradient fold (message_passing_op_cuda.py:75-93): grad_affinities
 * (N,4,K,H,W), each affinity the gradient of the taps it fills (L3: taps 1
 * and K+2), and grad_offset (N,4,H,W) = tap 0's.
 */
int bpl_unpack_tap_grad(const float* grad_taps, float* grad_affinities, float* grad_offset, int N, int K, int H,
                        int W, void* stream);

/*
 * dst (rows, Ls) half = sign * src (rows, L) float (sign +1 or -1), labels
 * L..Ls-1 zeroed, Ls = L rounded up to 8: the FP16-storage cost volume from
 * the layer's probability volume (cost = -prob, ops/lbp_stereo/
 * message_passing_op_cuda.py:162) in one pass.
 */
int bpl_half_padded(const float* src, float sign, void* dst, int64_t rows, int L, int Ls, void* stream);

/* Disparity count D of the SAD volume: (int)((max_disp - min_disp + 1) / step)
 * (ops/sad/src/stereo_sad_kernel.cu:122); -1 for a non-positive step. */
int bpl_sad_volume_depth(int min_disp, int max_disp, float step);

/*
 * Reference adjoint for FP16-stored messages (the layout of
 * bpl_lbp_forward_f16: label axis padded to Lp = L rounded up to 8).  No
 * counterpart in the reference.  in_grad and messages (B,4,H,W,Lp) half,
 * messages and scale as bpl_lbp_forward_f16 wrote them (min-referenced rows);
 * argmin (B,4,H,W,Lp); grad_cost (B,H,W,Lp) float (labels >= L are zero);
 * grad_jump / grad_edge as bpl_lbp_backward (float, unpadded).  workspace:
 * bpl_lbp_backward_workspace_size(B, H, W, Lp) bytes.  The normalisation's
 * Jacobian uses the softmax of each message row as it is now (the
 * reference's exp(m_raw)/S with m_raw rebuilt from the saved message and
 * log S is the softmax of the saved message, whichever pass S came from),
 * so scale is not read and may be NULL.  All variants.
 */
int bpl_lbp_backward_f16(int variant, const float* jump, const float* edge, const void* in_grad,
                         const void* messages, const void* argmin, int argmin_kind, const float* scale,
                         float* grad_cost, float* grad_jump, float* grad_edge, void* workspace,
                         size_t workspace_bytes, int B, int H, int W, int L, int Lv, int jump_batch,
                         int edge_batch, void* stream);

/*
 * Stereo SAD cost volume.  Replaces cuda::stereo_sad_forward
 * (ops/sad/src/stereo_sad_kernel.cu:116-136), bound as `forward`
 * (ops/sad/src/stereo_sad.cpp:10-15).
 * f0, f1 (B,C,H,W); out (B,H,W,D) with D = bpl_sad_volume_depth():
 * out[n,y,x,di] = sum over c in order of |f0[n,c,y,x] - f1[n,c,y,x-d]|,
 * d = (int)(di*step + min_disp), 40 where x-d is outside the image;
 * bit-identical to the reference.  For a fractional step the reference's
 * linear interpolation has weight 0 (d is an integer), so f1[x-d] is used.
 * At most 512 disparities.
 */
int bpl_sad_forward(const float* f0, const float* f1, float* out, int B, int C, int H, int W,
                    int min_disp, int max_disp, float step, void* stream);

/*
 * Gradient of the SAD volume (step 1).  Replaces cuda::stereo_sad_backward
 * (ops/sad/src/stereo_sad_kernel.cu:138-165), bound as `backward`
 * (ops/sad/src/stereo_sad.cpp:17-24).  in_grad (B,H,W,D); df0, df1 (B,C,H,W)
 * are zero-filled by this call.  Bit-identical to the reference.  With
 * reference_channel_limit != 0 only the first 4*ceil(D/4) channels receive a
 * gradient, as in the reference launch (:152-157); 0 covers all channels.
 */
int bpl_sad_backward(const float* f0, const float* f1, const float* in_grad, float* df0, float* df1,
                     int B, int C, int H, int W, int min_disp, int max_disp, int reference_channel_limit,
                     void* stream);

/*
 * Flow max-projected SAD.  Replaces cuda::flow_mp_sad_forward
 * (ops/flow_mp_sad/src/flow_mp_sad_kernel.cu:208-256), bound as `forward`
 * (ops/flow_mp_sad/src/flow_mp_sad.cpp:10-16).  f0, f1 (B,C,H,W); outputs
 * (B,H,W,K), K = sws+1: cv_u[u] = min over v of the window SAD, u_star[u] =
 * argmin_v + block_v*sws, cv_v[v] = min over u, v_star[v] = argmin_u +
 * block_u*sws (first index on ties; 40 outside the image); bit-identical to
 * the reference.  Windows up to K = 256 in one call (the reference's kernel
 * holds the K x K window in shared memory and stops at K = 128; its Python
 * layer merges four 108-windows for sws = 216, which equals one call here).
 */
int bpl_flow_forward(const float* f0, const float* f1, float* cv_u, float* cv_v, float* u_star,
                     float* v_star, int B, int C, int H, int W, int sws, int offset_u, int offset_v,
                     int block_u, int block_v, void* stream);

/*
 * Gradient of the flow SAD.  Replaces cuda::flow_mp_sad_backward
 * (ops/flow_mp_sad/src/flow_mp_sad_kernel.cu:258-290), bound as `backward`
 * (ops/flow_mp_sad/src/flow_mp_sad.cpp:18-30).  df0 is written (bit-identical
 * to the reference), df1 is accumulated with float atomics.  Like the
 * reference, offsets are not applied (correct for block 0, zero offsets).
 * The scratch (channel-last copies of f1 and df1) is allocated stream-ordered
 * (cudaMallocAsync) on `stream`; bpl_flow_backward_ws takes it from the
 * caller instead.
 */
int bpl_flow_backward(const float* f0, const float* f1, const float* in_grad_u, const float* in_grad_v,
                      const float* u_star, const float* v_star, float* df0, float* df1, int B, int C,
                      int H, int W, int sws, void* stream);

/* Scratch bytes bpl_flow_backward_ws needs: 2*B*C*H*W floats. */
size_t bpl_flow_backward_workspace_size(int B, int C, int H, int W);

/* bpl_flow_backward with caller-owned scratch (16-byte aligned, at least
 * bpl_flow_backward_workspace_size bytes; contents on entry are ignored). */
int bpl_flow_backward_ws(const float* f0, const float* f1, const float* in_grad_u, const float* in_grad_v,
                         const float* u_star, const float* v_star, float* df0, float* df1, void* workspace,
                         size_t workspace_bytes, int B, int C, int H, int W, int sws, void* stream);

/*
 * bpl_lbp_backward without device allocation.  No counterpart in the
 * reference (its backward allocates scratch with at::zeros on every step).
 * For hosts that cannot call cudaMalloc when they run the backward: device
 * memory owned by another runtime's pool, a fixed budget set at start-up, or
 * loops where an allocation's device synchronisation is not acceptable.
 * Arguments and results are those of bpl_lbp_backward minus the workspace:
 * the scratch is a fixed 16 MiB device array inside the library (held by
 * every GPU that loads it), so B*2*H*W*L*4 must not exceed 16 MiB
 * (BPL_ERR_INVALID_ARG otherwise).  All calls share that array: calls that
 * overlap on the GPU race and must be serialised by the caller.  The first
 * call on a device looks up the array's device address; make it before any
 * stream capture.  With CUDA's lazy module loading (the default) the array
 * comes into existence when the library's module is first loaded on a
 * device, which this call may trigger: that first call may allocate and
 * synchronise, so hosts that need every call allocation-free make one
 * warm-up call per device at start-up.  Only the device's primary context
 * (the runtime API's) is supported: the address is cached per device.
 */
int bpl_lbp_backward_noalloc(int variant, const float* jump, const float* edge, const float* in_grad,
                             const float* messages, const void* argmin, int argmin_kind,
                             const float* scale, float* grad_cost, float* grad_jump, float* grad_edge,
                             int B, int H, int W, int L, int Lv, int jump_batch, int edge_batch,
                             void* stream);

#ifdef __cplusplus
}
#endif

#endif /* BPL_GB300_H */
