/*
 * oracle.h -- CPU oracle for the checkers playout path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (libgpuai, the host
 * drivers, run_ai) links or calls this code.  Only tests/, the smoke check in
 * __graft_entry__.py and the cpu_baseline / reference leg of bench.py load it,
 * and only as the checker or as the timed CPU reference.
 *
 * It is a plain-C restatement of the reference's host algorithm (krame505/gpu_ai):
 *   - board / move types       src/state.hpp:10-26, 34-122, 253-296
 *   - move generation          src/state.cu:122-180, 239-245, 255-340, 388-420, 456-462
 *   - applying a move          src/state.cu:46-92
 *   - terminal test / winner   src/state.cpp:10-23
 *   - start position           src/state.cpp:25-40
 *   - heuristic                src/heuristic.cu:7-49, src/heuristic.hpp:5-8
 *   - host playout drivers     src/playout.cpp:17-32, src/player.cpp:13-16,
 *                              src/heuristicPlayout.cpp:12-48
 * plus the project's own random streams (Philox4x32-10, Salmon et al., SC'11)
 * so that every GPU playout can be replayed move by move on the CPU.
 *
 * Parity pin: the restatement is checked move-list-exact against the
 * reference's own State::genMoves and against HostPlayoutDriver outcome
 * frequencies (tests/test_oracle_pin.py builds the reference from its
 * sources into oracle/_ref/ where they are present) and against golden
 * vectors generated from the reference (tests/golden/).
 */
#ifndef GPUAI_ORACLE_H
#define GPUAI_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Reference limits are MAX_MOVE_JUMPS 8 and MAX_MOVES 100 (state.hpp:17-19);
 * the restatement keeps larger arrays so that it never overflows where the
 * reference would. */
#define OR_MAX_JUMPS 16
#define OR_MAX_MOVES 160
#define OR_DRAW_PLIES 50 /* NUM_DRAW_MOVES, state.hpp:14 */

enum { OR_P1 = 0, OR_P2 = 1, OR_NONE = -1 };  /* PlayerId, state.hpp:21-26 */
enum { OR_MAN = 0, OR_KING = 1 };            /* PieceType, state.hpp:28-31 */

typedef struct { uint8_t occupied, type; int8_t owner; } or_item;   /* BoardItem */
typedef struct { int8_t r, c; } or_loc;                              /* Loc */
typedef struct { or_item board[8][8]; int32_t turn; uint32_t msc; } or_state; /* State */
typedef struct {
  or_loc from, to;
  or_loc removed[OR_MAX_JUMPS];
  or_loc inter[OR_MAX_JUMPS];
  uint8_t jumps, promoted;
} or_move;                                                           /* Move */

/* 16-byte bitboard record shared with the product ABI (include/gpuai.h):
 * square s = row*4 + col/2 over the 32 dark squares. */
typedef struct { uint32_t p1, p2, kings, meta; } or_board16;

/* 32-byte packed move shared with the product ABI (gpuai_move). */
typedef struct {
  uint8_t from, to, jumps, promoted;
  uint8_t path[12];    /* landing squares in order ("intermediate", incl. final) */
  uint8_t removed[12]; /* captured squares in order */
  uint8_t pad[4];
} or_packed_move;

/* ---- board conversion ---- */
void or_from_board16(const or_board16 *b, or_state *s);
void or_to_board16(const or_state *s, or_board16 *b);
void or_start_state(or_state *s);
void or_pack_move(const or_move *m, or_packed_move *out);

/* ---- rules (reference restatement) ---- */
int or_genmoves(const or_state *s, or_move *result);      /* State::genMoves */
void or_apply(or_state *s, const or_move *m);             /* State::move */
int or_is_over(const or_state *s);                        /* State::isGameOver */
int or_winner(const or_state *s);                         /* State::getWinner */

/* batch helpers over board16 arrays (ctypes friendly) */
int or_genmoves_b16(const or_board16 *pos, uint32_t n, or_packed_move *out,
                    uint32_t max_moves, uint8_t *counts);
int or_apply_packed_b16(or_board16 *pos, const or_packed_move *m);

/* ---- heuristic (heuristic.cu:7-49) ---- */
void or_score_state(const or_state *s, unsigned score[2]);
void or_score_move(const or_state *s, const or_move *m, int score[2]);
float or_get_weight(const or_state *s, const unsigned ss[2], const int ms[2]);

/* ---- project random streams: Philox4x32-10 ---- */
void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* draw k of the stream (seed, id, tag): word k&3 of
 * philox(ctr = {k>>2, id_lo, id_hi, tag}, key = {seed_lo, seed_hi}) */
uint32_t or_stream_draw(uint64_t seed, uint64_t id, uint32_t tag, uint32_t k);

/* ---- replay harness: one playout, move list in reference order ---- */
/* policy 0 = uniform random.  Returns outcome (+1 P1 won, -1 P2 won, 0 draw);
 * *plies = plies played, *draws = random draws consumed. */
int or_replay_playout(const or_board16 *pos, uint64_t seed, uint64_t id, int policy,
                      uint32_t *plies, uint32_t *draws);
void or_replay_batch(const or_board16 *pos, const uint32_t *reps, uint32_t npos,
                     uint64_t seed, uint64_t stream_base, int policy, int8_t *out,
                     uint32_t *plies, int nthreads);

/* seeded positions: position p applies U{min..max} random plies from the start */
void or_random_positions(uint64_t seed, uint32_t n, uint32_t min_plies, uint32_t max_plies,
                         or_board16 *out);

/* ---- reference host drivers, restated (CPU baseline "port") ---- */
/* HostPlayoutDriver::runPlayouts: OpenMP over states, rand() % n per ply. */
void or_host_playouts(const or_board16 *states, uint32_t n, int8_t *out, int nthreads,
                      unsigned srand_seed);
/* HostHeuristicPlayoutDriver::runPlayouts: argmax of heuristic weight plus
 * N(0, 0.11) noise, the move list generated twice per ply, the noise drawn
 * from one minstd engine shared by all OpenMP threads as in the reference.
 * A restatement of the reference's cost structure; its outcomes agree with the
 * reference's in distribution only. */
void or_host_heuristic_playouts(const or_board16 *states, uint32_t n, int8_t *out,
                                uint64_t seed);

#ifdef __cplusplus
}
#endif
#endif
