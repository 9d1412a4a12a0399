/*
 * gpuai.h -- C ABI of the GB300 checkers playout engine (libgpuai.so).
 *
 * Plain C types only: no CUDA or C++ types cross this boundary.  Every call
 * returns a status (GPUAI_OK or a negative GPUAI_ERR_*); none exits the
 * process.  gpuai_last_error() gives the message of the calling thread's last
 * failure.
 *
 * Boards are 16-byte bitboard records over the 32 dark squares, square
 * s = row*4 + col/2 (row 0 is PLAYER_1's back rank, dark squares are
 * col = 1-(row%2), +2, ...).  Outcomes are int8: +1 PLAYER_1 won, -1 PLAYER_2
 * won, 0 drawn.
 *
 * Threading: calls on one context are serialised by the context; use one
 * context per host thread (each owns its own CUDA stream) for concurrency.
 */
#ifndef GPUAI_H
#define GPUAI_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GPUAI_OK 0
#define GPUAI_ERR_INVALID (-1)   /* bad argument or malformed board */
#define GPUAI_ERR_CUDA (-2)      /* CUDA runtime error (message says which) */
#define GPUAI_ERR_OOM (-3)       /* device or pinned allocation failed */
#define GPUAI_ERR_LIMIT (-4)     /* a kernel hit an internal limit (status word) */
#define GPUAI_ERR_NO_DEVICE (-5) /* no CUDA device, or the device index is out of range */

#define GPUAI_POLICY_RANDOM 0        /* uniform over the legal move list */
#define GPUAI_POLICY_REF_HEURISTIC 1 /* argmax of material-ratio weight + noise */
#define GPUAI_POLICY_EPS_GREEDY 2    /* eps = 0.1 random, else greedy material+advancement */

/* Board record.  meta: bit 0 = side to move (0 PLAYER_1, 1 PLAYER_2);
 * bits 8..15 = plies since the last capture (>= 50 is a draw); other bits 0. */
typedef struct gpuai_board {
  uint32_t p1;    /* squares holding PLAYER_1 pieces */
  uint32_t p2;    /* squares holding PLAYER_2 pieces */
  uint32_t kings; /* squares holding kings (either side) */
  uint32_t meta;
} gpuai_board;

/* One legal move, 32 bytes.  Unused path/removed slots are 0xFF. */
typedef struct gpuai_move {
  uint8_t from, to, jumps, promoted;
  uint8_t path[12];    /* landing square of each jump, in order (last = to) */
  uint8_t removed[12]; /* captured square of each jump, in order */
  uint8_t pad[4];      /* zero */
} gpuai_move;

typedef struct gpuai_ctx gpuai_ctx;

/* Create a context on CUDA device `device` with its own stream.
 * Replaces the per-call cudaMalloc/stack-limit set-up of
 * DeviceMultiplePlayoutDriver::runPlayouts (src/multiplePlayout.cu:53-98). */
int gpuai_create(int device, gpuai_ctx **out);
void gpuai_destroy(gpuai_ctx *ctx);

/* Message of the calling thread's last failed call ("" if none). */
const char *gpuai_last_error(void);

/* Run playouts from host buffers: reps[p] playouts from pos[p] (reps NULL
 * means one each), outcomes written in order to out (sum of reps entries).
 * Playout j (0-based over the whole call) uses random stream id
 * stream_base + j under `seed`.  npos == 0 returns GPUAI_OK without a launch.
 * Replaces PlayoutDriver::runPlayouts (src/playout.hpp:27-33) as implemented
 * by DeviceMultiplePlayoutDriver / DeviceSinglePlayoutDriver /
 * DeviceCoarsePlayoutDriver / DeviceHeuristicPlayoutDriver
 * (src/multiplePlayout.cu:53-98, src/singlePlayout.cu:71-120,
 * src/coarsePlayout.cu:91-163, src/heuristicPlayout.cu:102-147). */
int gpuai_playouts(gpuai_ctx *ctx, const gpuai_board *pos, const uint32_t *reps, uint32_t npos,
                   uint64_t seed, uint64_t stream_base, int32_t policy, int8_t *out);

/* Same work on device-resident buffers, enqueued on `stream` (a cudaStream_t;
 * NULL is the legacy default stream) without synchronising.  d_offsets holds
 * npos+1 exclusive prefix sums of the repetitions, or is NULL when every
 * position has `uniform_reps` playouts.  total = number of playouts.  Calls on
 * one context must be ordered on one stream: they share the context's work
 * counter.  Check gpuai_status() after synchronising. */
int gpuai_playouts_device(gpuai_ctx *ctx, const gpuai_board *d_pos, const uint32_t *d_offsets,
                          uint32_t npos, uint32_t uniform_reps, uint32_t total, uint64_t seed,
                          uint64_t stream_base, int32_t policy, int8_t *d_out, void *stream);

/* Status word and ply count of the context's last playout call, host-buffer
 * or device-side (synchronises the device first).  status 0 = fine. */
int gpuai_status(gpuai_ctx *ctx, uint32_t *status, uint64_t *plies);

/* Legal move lists of n boards, in the reference's State::genMoves order
 * (src/state.cu:239-245): out[i*max_moves + k], counts[i] = number of moves.
 * Returns GPUAI_ERR_LIMIT if some list is longer than max_moves. */
int gpuai_genmoves(gpuai_ctx *ctx, const gpuai_board *pos, uint32_t n, gpuai_move *out,
                   uint32_t max_moves, uint8_t *counts);

/* n seeded positions: position i plays U{min_plies..max_plies} uniformly random
 * legal plies from the standard start (stopping early at a finished game).
 * Replaces genRandomStates (src/driver.cpp:76-104). */
int gpuai_random_positions(gpuai_ctx *ctx, uint64_t seed, uint32_t n, uint32_t min_plies,
                           uint32_t max_plies, gpuai_board *out);

/* Device-side variant for training data: n positions into d_out (device),
 * position i after U{min_plies..max_plies} plies of `policy` (GPUAI_POLICY_*)
 * from the standard start, stopping early at a finished game; enqueued on
 * `stream` (NULL = legacy default stream).  With GPUAI_POLICY_RANDOM the
 * positions equal gpuai_random_positions' for the same seed. */
int gpuai_selfplay_positions(gpuai_ctx *ctx, uint64_t seed, uint32_t n, uint32_t min_plies, uint32_t max_plies,
                             int32_t policy, gpuai_board *d_out, void *stream);

/* Host-side State::move (src/state.cu:57-92): the board after `move`, a
 * record of the board's legal move list (gpuai_genmoves).  Needs no context
 * or device. */
int gpuai_apply_move(const gpuai_board *board, const gpuai_move *move, gpuai_board *out);

/* Number of SMs, and the launch shape of the uniform-random playout kernel. */
int gpuai_device_info(gpuai_ctx *ctx, int32_t *sms, int32_t *blocks_per_sm, int32_t *block_threads);

/* Launch shape of the playout kernel for `policy`: threads per block (64,
 * 128, 256 or 512) and resident blocks per SM the persistent grid uses
 * (0 = as many as fit).  The grid is SMs x blocks_per_sm, or fewer blocks for
 * small batches.  Results do not depend on the launch shape.  This is the
 * knob the autotuner sweeps; it has no counterpart in the reference, whose
 * drivers hard-code <<<N,32>>>, <<<N/128,128>>> and the coarse grid
 * (src/multiplePlayout.cu:77, src/singlePlayout.cu:86-99, src/coarsePlayout.cu:113-115). */
int gpuai_set_launch(gpuai_ctx *ctx, int32_t policy, int32_t block_threads, int32_t blocks_per_sm);
int gpuai_get_launch(gpuai_ctx *ctx, int32_t policy, int32_t *block_threads, int32_t *blocks_per_sm,
                     int32_t *max_blocks_per_sm);

/* Playout layout for `policy`: a thread per playout (GPUAI_LAYOUT_THREAD, the
 * default, every policy), a warp per playout with one lane per dark square
 * (GPUAI_LAYOUT_WARP, uniform random policy only), the shape of the
 * reference's playoutKernel (src/multiplePlayout.cu:14-52), or a thread per
 * playout whose plies that must search a multi-jump are handed to a block-wide
 * pool and played by full warps (GPUAI_LAYOUT_POOLED, every policy).  Outcomes
 * are the same in all layouts; the autotuner measures which is faster.
 * Setting a layout resets blocks_per_sm to as many as fit. */
#define GPUAI_LAYOUT_THREAD 0
#define GPUAI_LAYOUT_WARP 1
#define GPUAI_LAYOUT_POOLED 2
int gpuai_set_layout(gpuai_ctx *ctx, int32_t policy, int32_t layout);
int gpuai_get_layout(gpuai_ctx *ctx, int32_t policy, int32_t *layout);

/* ---- many searches with device-resident trees ----
 * Replaces the reference's one-search-per-MCTSPlayer loop
 * (src/player.cpp:134-150, src/mcts.cpp:63-191) with searches whose UCT trees
 * live in one node pool in device memory.  One step advances every active
 * search: `leaves_per_search` leaf slots per search are split over its tree
 * level by level with the reference's GameTree::select rule (a leaf given
 * more than one slot is expanded), playouts_per_leaf GPU playouts per leaf,
 * and backpropagation; the step's kernels can be replayed as a CUDA graph.
 * A search's result does not depend on the other searches it shares steps
 * with.  Best move = most visited root child. */
typedef struct gpuai_searches gpuai_searches;

/* pool_nodes: node capacity of the shared pool (52 bytes of device memory per
 * node); max_leaves_per_step (at most 512) bounds leaves_per_search. */
int gpuai_searches_create(int device, uint32_t max_searches, uint32_t pool_nodes, uint32_t max_leaves_per_step,
                          uint32_t playouts_per_leaf, int32_t policy, uint64_t seed, gpuai_searches **out);
void gpuai_searches_destroy(gpuai_searches *s);
/* Admit a search from `root` that stops after `playout_budget` playouts and
 * may grow to `node_capacity` nodes; its playouts use random stream ids from
 * stream_base on.  GPUAI_ERR_OOM = admission refused (no free slot or no free
 * node range of that size). */
int gpuai_searches_add(gpuai_searches *s, const gpuai_board *root, uint64_t playout_budget, uint32_t node_capacity,
                       uint64_t stream_base, int32_t *slot);
int gpuai_searches_remove(gpuai_searches *s, int32_t slot);
/* Enqueue `steps` steps (no synchronisation). */
int gpuai_searches_step(gpuai_searches *s, uint32_t steps, uint32_t leaves_per_search, int32_t use_graph);
/* Synchronise; playouts done and budget of slots 0..n-1 (0 for free slots). */
int gpuai_searches_poll(gpuai_searches *s, uint64_t *done, uint64_t *budget, uint32_t n, uint32_t *status);
/* Root children of a search: moves (reference move-list order), visits and
 * score in half points for the player to move at the root. */
int gpuai_searches_children(gpuai_searches *s, int32_t slot, gpuai_move *moves, uint32_t *visits,
                            uint32_t *score2, uint32_t max_children, uint32_t *nchildren, uint32_t *nodes_used);

/* Learned searches whose playouts are learned-proposal playouts
 * (gpuai_playouts_learned): the first guided_plies plies of every playout are
 * drawn from the attached network's policy at `temperature` (0 turns it off:
 * plain playouts of the searches' policy).  The first guided ply uses the
 * forward pass on the leaves that also gives the priors and leaf values; later
 * ones run the network on the playouts' boards.  Needs a network attached and
 * no admitted searches. */
int gpuai_searches_set_proposal(gpuai_searches *s, uint32_t guided_plies, float temperature);

/* Inspection of the device trees, for tests and tools (no counterpart in the
 * reference, whose GameTree keeps its nodes private).  Synchronise first.
 * gpuai_searches_nodes: the first min(nnodes, max_nodes) nodes of the search in
 * `slot`, numbered from its root (0) in allocation order; *nnodes = nodes in
 * use.  info (optional, 4 words per node): first child (0xFFFFFFFF before
 * expansion), children | state bits << 16 (1 expanded, 2 finished root,
 * 4 evaluated by the network), playouts through the node (visit units for
 * learned searches), score in half points of the player who moved into the
 * node.  boards, parent (-1 for the root) and priors (32 FP16 bit patterns
 * per node, learned searches only) are optional too. */
int gpuai_searches_nodes(gpuai_searches *s, int32_t slot, uint32_t max_nodes, uint32_t *info, gpuai_board *boards,
                         int32_t *parent, uint16_t *priors, uint32_t *nnodes);
/* The last step's leaf slots, in slot order (searches in slot order, each
 * search's slots in the order its selection emitted them); *nleaves = their
 * number.  Per slot (all optional): search slot, node (numbered from the
 * search's root), board, first random-stream id (its playouts use that id and
 * the next playouts_per_leaf - 1), outcomes (playouts_per_leaf int8 each) and,
 * with a network attached, its raw value output (before tanh) and 1024 BF16
 * move logits (bit patterns). */
int gpuai_searches_leaves(gpuai_searches *s, uint32_t max_leaves, uint32_t *nleaves, int32_t *search, int32_t *node,
                          gpuai_board *boards, uint64_t *streams, int8_t *outcomes, float *net_value,
                          uint16_t *net_logits);

/* ---- policy/value network ----
 * No counterpart in the reference (its only evaluation is the material
 * heuristic, src/heuristic.cu:20-49).  A BF16 MLP on the tensor cores with FP32
 * accumulation: 129 input features (side to move's men, its kings, the
 * opponent's men, its kings, 32 squares each, then 1 if PLAYER_2 is to move),
 * two hidden layers of 256 ReLU units, 1024 move logits (index from*32 + to,
 * masked to the legal moves by the caller) and a tanh value for the side to
 * move.  Parameters, FP32, in this order (GPUAI_NET_PARAMS floats):
 *   W1[256][192] (input features 129..191 are zero padding), b1[256],
 *   W2[256][256], b2[256], W3[1024][256], b3[1024], wv[256], bv[1].
 * Forward, backward and Adam run as the library's own kernels; the GEMMs use
 * BF16 copies of W1..W3 and BF16 activations.  Training targets per position:
 * the value z for the side to move in [-1, 1], and move_q[32]: the value of
 * each legal move (reference move-list order) for the side to move; the
 * policy target is softmax(move_q / tau) over the legal moves.  Loss per
 * position = cross entropy(policy target, masked softmax of the logits)
 * + value_coef * (tanh value - z)^2, averaged over the batch.  Positions with
 * more than GPUAI_NET_MAX_MOVES legal moves train the value only. */
#define GPUAI_NET_FEATURES 129
#define GPUAI_NET_HIDDEN 256
#define GPUAI_NET_LOGITS 1024
#define GPUAI_NET_MAX_MOVES 32
#define GPUAI_NET_PARAMS 378625
typedef struct gpuai_net gpuai_net;

/* Parameters initialised uniformly in +-sqrt(6 / (fan_in + fan_out)) from
 * Philox stream (init_seed), biases 0; max_batch = largest training batch. */
int gpuai_net_create(int device, uint32_t max_batch, uint64_t init_seed, gpuai_net **out);
void gpuai_net_destroy(gpuai_net *net);
/* Host copies of the FP32 parameters; set_params also clears Adam's state. */
int gpuai_net_get_params(gpuai_net *net, float *params);
int gpuai_net_set_params(gpuai_net *net, const float *params);
/* Parameters and Adam state as little-endian FP32 after a 64-byte header. */
int gpuai_net_save(gpuai_net *net, const char *path);
int gpuai_net_load(gpuai_net *net, const char *path);
/* Forward pass on host boards: value[n] = tanh value for the side to move;
 * logits (optional) = n x 1024 raw move logits. */
int gpuai_net_forward(gpuai_net *net, const gpuai_board *boards, uint32_t n, float *value, float *logits);
/* Gradients of the loss (host buffers, n <= max_batch) without an update:
 * grads[GPUAI_NET_PARAMS] in parameter order; loss2 = {policy, value} means. */
int gpuai_net_gradients(gpuai_net *net, const gpuai_board *boards, const float *value_target,
                        const float *move_q, uint32_t n, float tau, float value_coef, float *grads,
                        float *loss2);
/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8) on device-resident
 * training rows d_boards[n], d_value_target[n], d_move_q[n*32], enqueued on the
 * net's stream.  The step's kernels read the rows in place: leave them
 * unchanged until the net's stream has run the step; d_boards must be 16-byte
 * aligned, the others 4-byte (GPUAI_ERR_INVALID otherwise).  loss2 (host,
 * optional) makes the call wait and return the step's mean policy and value
 * losses. */
int gpuai_net_train_step(gpuai_net *net, const gpuai_board *d_boards, const float *d_value_target,
                         const float *d_move_q, uint32_t n, float lr, float tau, float value_coef, float *loss2);
/* Training labels from GPU playouts, on device buffers: for each position,
 * each legal move m gets playouts_per_position / k (+1 for the first
 * playouts_per_position % k moves) playouts of `policy` from the position after
 * m; d_move_q[i*32 + m] = their mean outcome for the side to move at position
 * i, d_value[i] = the mean over all its playouts (a random first move then
 * playouts: the same estimate as that many playouts from position i).
 * d_nmoves[i] = k, or 0 when the game is over or k > 32 (values then 0).
 * Playout j of position i uses stream id stream_base + i * playouts_per_position
 * + j under `seed`.  Enqueued on `stream` (NULL = legacy default stream);
 * n * playouts_per_position must stay below 2^31. */
int gpuai_label_positions(gpuai_ctx *ctx, const gpuai_board *d_pos, uint32_t n, uint32_t playouts_per_position,
                          uint64_t seed, uint64_t stream_base, int32_t policy, float *d_value, float *d_move_q,
                          uint8_t *d_nmoves, void *stream);
/* Self-test of the tensor-core kernels' bounded waits (no counterpart in the
 * reference): one tile of the first layer's GEMM is launched with no TMA load
 * issued and every barrier wait limited to wait_limit_us (1..10^6), so the
 * MMA warp's wait for its first stage runs out.  The kernel then records the
 * failure in the status word, frees its tensor memory and returns; *status is
 * that word (bit 16 set when the wait ran out), cleared afterwards.  The
 * network stays usable. */
int gpuai_net_wait_selftest(gpuai_net *net, uint32_t wait_limit_us, uint32_t *status);

/* Learned-proposal playouts (no counterpart in the reference; the shape of its
 * heuristicPlayoutKernel, src/heuristicPlayout.cu:54-88, with the network's
 * policy in place of scoreMove): the first guided_plies plies of every playout
 * are drawn from the network's policy -- the softmax at `temperature` of each
 * legal move's (from, to) logit over the legal pairs, a pair's share split
 * equally among the moves that have it, as integer weights
 * max(1, floor(2^24 e^((l - lmax) / T)) / multiplicity) -- and the rest of the
 * game is uniformly random (GPUAI_POLICY_RANDOM), the fallback and judge of the
 * network.  Guided ply g of playout j takes draw g of random stream
 * (seed, stream_base + j, tag 2); its random plies use stream
 * (seed, stream_base + j, tag 0) from the board after the guided plies, as
 * gpuai_playouts does.  Device buffers as gpuai_playouts_device, enqueued on
 * `stream` without synchronising; guided_plies == 0 is plain random playouts,
 * at most 32.  The network keeps a workspace sized for the largest call so far
 * (growing it synchronises the device).  d_trace_boards / d_trace_logits
 * (optional, device, guided_plies * total entries: boards, and 1024 BF16 bit
 * patterns each) receive each playout's board before every guided ply and the
 * logits it was drawn from, for tests that replay the choices. */
int gpuai_playouts_learned(gpuai_ctx *ctx, gpuai_net *net, const gpuai_board *d_pos, const uint32_t *d_offsets,
                           uint32_t npos, uint32_t uniform_reps, uint32_t total, uint64_t seed, uint64_t stream_base,
                           uint32_t guided_plies, float temperature, int8_t *d_out, void *stream,
                           gpuai_board *d_trace_boards, uint16_t *d_trace_logits);

/* Learned searches: leaves are also evaluated by `net` (NULL turns it off).
 * Each leaf's value is value_weight * net value + (1 - value_weight) * its
 * playout mean; a node's moves get the net's softmax over its legal moves as
 * priors once it has been a leaf, and slots are split with PUCT
 * (Q + c_puct * P * sqrt(N) / (1 + n)) instead of UCB1.  The net must not be
 * trained while searches use it. */
int gpuai_searches_set_net(gpuai_searches *s, gpuai_net *net, float value_weight, float c_puct);

/* Playouts that allocate no device memory, for callers that may not call
 * cudaMalloc: for example a search server that reserves the whole device
 * memory budget for its trees up front, or a move loop with a hard per-move
 * deadline that must never wait on the allocator.  It has no counterpart in
 * the reference.  d_pos (npos boards) and d_out (one int8 outcome per playout)
 * are device buffers the caller already owns; reps is a HOST array of
 * repetitions (NULL: one playout per board); results equal gpuai_playouts with
 * the same seed and stream_base.  The work counter, status word and the
 * repetition prefix sums live in one statically allocated device array per
 * GPU, sized for at most GPUAI_NOALLOC_MAX_POSITIONS positions (about 64 KiB,
 * held until the process exits); larger npos is rejected with
 * GPUAI_ERR_INVALID.  No context is needed: the call runs on the current
 * device and `stream` (NULL: the legacy default stream) and returns after the
 * playouts finished: every call synchronises `stream` before it returns.  The
 * first call on a device looks up that array's device address; make that
 * first call before any stream capture.  All calls share the array,
 * which keeps the previous call's contents (the call clears what must start
 * at zero); calls on one device are serialised by the library, and launches
 * that overlapped on the GPU would race on it. */
#define GPUAI_NOALLOC_MAX_POSITIONS 16384
int gpuai_playouts_noalloc(const gpuai_board *d_pos, const uint32_t *reps, uint32_t npos,
                           uint64_t seed, uint64_t stream_base, int32_t policy, int8_t *d_out,
                           void *stream);

#ifdef __cplusplus
}
#endif
#endif /* GPUAI_H */
