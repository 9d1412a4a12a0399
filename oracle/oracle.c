/*
 * oracle.c -- CPU oracle for the checkers playout path (TEST INFRASTRUCTURE).
 *
 * Restates the reference's host algorithm function by function; every
 * function cites the reference file:line it follows.  The product never links
 * this file.  See oracle.h for the parity pins.
 */
#include "oracle.h"

#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <stdatomic.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* board helpers                                                        */
/* ------------------------------------------------------------------ */

static inline int loc_valid(int r, int c) { return r >= 0 && r < 8 && c >= 0 && c < 8; }
static inline int loc_sq(or_loc l) { return l.r * 4 + l.c / 2; }
static inline or_loc mkloc(int r, int c) { or_loc l; l.r = (int8_t)r; l.c = (int8_t)c; return l; }
static inline int loc_eq(or_loc a, or_loc b) { return a.r == b.r && a.c == b.c; }

static inline void sq_to_rc(int sq, int *r, int *c) {
  *r = sq >> 2;
  *c = 2 * (sq & 3) + ((*r & 1) ? 0 : 1); /* dark squares: col = 1-(row%2), +2 ... (state.cu:174) */
}

void or_from_board16(const or_board16 *b, or_state *s) {
  memset(s, 0, sizeof(*s));
  for (int sq = 0; sq < 32; sq++) {
    int r, c;
    sq_to_rc(sq, &r, &c);
    uint32_t bit = 1u << sq;
    or_item *it = &s->board[r][c];
    if (b->p1 & bit) { it->occupied = 1; it->owner = OR_P1; }
    else if (b->p2 & bit) { it->occupied = 1; it->owner = OR_P2; }
    if (it->occupied) it->type = (b->kings & bit) ? OR_KING : OR_MAN;
  }
  s->turn = (b->meta & 1u) ? OR_P2 : OR_P1;
  s->msc = (b->meta >> 8) & 0xffu;
}

void or_to_board16(const or_state *s, or_board16 *b) {
  memset(b, 0, sizeof(*b));
  for (int sq = 0; sq < 32; sq++) {
    int r, c;
    sq_to_rc(sq, &r, &c);
    const or_item *it = &s->board[r][c];
    if (!it->occupied) continue;
    if (it->owner == OR_P1) b->p1 |= 1u << sq; else b->p2 |= 1u << sq;
    if (it->type == OR_KING) b->kings |= 1u << sq;
  }
  uint32_t msc = s->msc > 255u ? 255u : s->msc;
  b->meta = (s->turn == OR_P2 ? 1u : 0u) | (msc << 8);
}

/* getStartingState (state.cpp:25-40): P1 men on rows 0-2, P2 men on rows
 * 5-7, P1 to move, counter 0. */
void or_start_state(or_state *s) {
  memset(s, 0, sizeof(*s));
  for (int r = 0; r < 8; r++)
    for (int c = 1 - (r % 2); c < 8; c += 2) {
      if (r <= 2) { s->board[r][c].occupied = 1; s->board[r][c].owner = OR_P1; }
      if (r >= 5) { s->board[r][c].occupied = 1; s->board[r][c].owner = OR_P2; }
    }
  s->turn = OR_P1;
  s->msc = 0;
}

void or_pack_move(const or_move *m, or_packed_move *out) {
  memset(out, 0xff, sizeof(*out));
  out->from = (uint8_t)loc_sq(m->from);
  out->to = (uint8_t)loc_sq(m->to);
  out->jumps = m->jumps;
  out->promoted = m->promoted ? 1 : 0;
  for (int i = 0; i < m->jumps && i < 12; i++) {
    out->path[i] = (uint8_t)loc_sq(m->inter[i]);
    out->removed[i] = (uint8_t)loc_sq(m->removed[i]);
  }
  out->pad[0] = out->pad[1] = out->pad[2] = out->pad[3] = 0;
}

/* ------------------------------------------------------------------ */
/* move generation (state.cu)                                           */
/* ------------------------------------------------------------------ */

static inline const or_item *at(const or_state *s, or_loc l) { return &s->board[l.r][l.c]; }

static inline int next_turn(int t) { return t == OR_P1 ? OR_P2 : (t == OR_P2 ? OR_P1 : OR_NONE); }

static void move_init(or_move *m, or_loc from, or_loc to, int jumps, int promoted) {
  m->from = from; m->to = to; m->jumps = (uint8_t)jumps; m->promoted = (uint8_t)promoted;
}

/* Move::addJump (state.cu:456-462) */
static void move_add_jump(or_move *m, or_loc nt) {
  m->inter[m->jumps] = nt;
  m->removed[m->jumps] = mkloc((nt.r - m->to.r) / 2 + m->to.r, (nt.c - m->to.c) / 2 + m->to.c);
  m->jumps++;
  m->to = nt;
}

/* State::isValidJump (state.cu:122-142) */
static int is_valid_jump(const or_state *s, const or_move *m, int jr, int jc, int tr, int tc,
                         int check_cycles) {
  if (!loc_valid(tr, tc) || !loc_valid(jr, jc)) return 0;
  const or_item *j = &s->board[jr][jc];
  if (!j->occupied || j->owner == s->turn || s->board[tr][tc].occupied) return 0;
  if (check_cycles)
    for (int i = m->jumps - 1; i >= 0; i--)
      if (m->inter[i].r == tr && m->inter[i].c == tc) return 0;
  return 1;
}

/* State::genLocDirectMoves (state.cu:255-281): kings try (dr,dc) =
 * (+1,+1),(+1,-1),(-1,+1),(-1,-1); men only the forward pair. */
static int gen_loc_direct(const or_state *s, or_loc loc, or_move *result) {
  static const int dc[] = {1, -1, 1, -1};
  static const int dr[] = {1, 1, -1, -1};
  int count = 0;
  const or_item *it = at(s, loc);
  if (it->type == OR_KING) {
    for (int i = 0; i < 4; i++) {
      int r = loc.r + dr[i], c = loc.c + dc[i];
      if (loc_valid(r, c) && !s->board[r][c].occupied)
        move_init(&result[count++], loc, mkloc(r, c), 0, 0);
    }
  } else {
    int start = it->owner == OR_P1 ? 0 : 2, end = it->owner == OR_P1 ? 2 : 4;
    for (int i = start; i < end; i++) {
      int r = loc.r + dr[i], c = loc.c + dc[i];
      if (loc_valid(r, c) && !s->board[r][c].occupied)
        move_init(&result[count++], loc, mkloc(r, c), 0,
                  r == (it->owner == OR_P1 ? 7 : 0));
    }
  }
  return count;
}

/* State::genLocCaptureReg (state.cu:283-340): DFS, left (dc=-1) before right
 * (dc=+1), forward only; a sequence is emitted only when no further jump
 * exists; promoted if the final square is the far row.  The board is not
 * updated during the search. */
static int gen_loc_capture_reg(const or_state *s, or_loc loc, or_move *result, int count, int first) {
  or_move prev = result[count];
  int dRL, dCL, dRR, dCR;
  if (at(s, result[0].from)->owner == OR_P1) { dRL = 1; dCL = -1; dRR = 1; dCR = 1; }
  else { dRL = -1; dCL = -1; dRR = -1; dCR = 1; }
  int jlr = loc.r + dRL, jlc = loc.c + dCL, jrr = loc.r + dRR, jrc = loc.c + dCR;
  int tlr = loc.r + 2 * dRL, tlc = loc.c + 2 * dCL, trr = loc.r + 2 * dRR, trc = loc.c + 2 * dCR;
  int left = is_valid_jump(s, &result[count], jlr, jlc, tlr, tlc, 0);
  int right = is_valid_jump(s, &result[count], jrr, jrc, trr, trc, 0);
  if (!left && !right && !first) {
    if (s->turn == OR_P1 && result[count].to.r == 7) result[count].promoted = 1;
    if (s->turn == OR_P2 && result[count].to.r == 0) result[count].promoted = 1;
    return count + 1;
  }
  if (left) {
    result[count] = prev;
    move_add_jump(&result[count], mkloc(tlr, tlc));
    count = gen_loc_capture_reg(s, mkloc(tlr, tlc), result, count, 0);
  }
  if (right) {
    result[count] = prev;
    move_add_jump(&result[count], mkloc(trr, trc));
    count = gen_loc_capture_reg(s, mkloc(trr, trc), result, count, 0);
  }
  return count;
}

/* State::genLocCaptureKing (state.cu:388-420): DFS in direction order
 * (+1,+1),(+1,-1),(-1,+1),(-1,-1) with the landing-square cycle check. */
static int gen_loc_capture_king(const or_state *s, or_loc loc, or_move *result, int count, int first) {
  static const int dR[4] = {1, 1, -1, -1};
  static const int dC[4] = {1, -1, 1, -1};
  or_move prev = result[count];
  or_loc to[4];
  int valid[4];
  for (int i = 0; i < 4; i++) {
    to[i] = mkloc(loc.r + 2 * dR[i], loc.c + 2 * dC[i]);
    valid[i] = is_valid_jump(s, &prev, loc.r + dR[i], loc.c + dC[i], to[i].r, to[i].c, 1);
  }
  if (!first && !(valid[0] | valid[1] | valid[2] | valid[3])) return count + 1;
  for (int i = 0; i < 4; i++)
    if (valid[i]) {
      result[count] = prev;
      move_add_jump(&result[count], to[i]);
      count = gen_loc_capture_king(s, to[i], result, count, 0);
    }
  return count;
}

/* State::genLocMoves (state.cu:144-169) for DIRECT (0) and CAPTURE (1). */
static int gen_loc_moves(const or_state *s, or_loc loc, or_move *result, int capture) {
  const or_item *it = at(s, loc);
  if (!it->occupied || it->owner != s->turn) return 0;
  if (!capture) return gen_loc_direct(s, loc, result);
  move_init(&result[0], loc, loc, 0, 0);
  if (it->type == OR_MAN) return gen_loc_capture_reg(s, loc, result, 0, 1);
  return gen_loc_capture_king(s, loc, result, 0, 1);
}

/* State::genTypeMoves (state.cu:171-180): row-major over the dark squares. */
static int gen_type_moves(const or_state *s, or_move *result, int capture) {
  int n = 0;
  for (int i = 0; i < 8; i++)
    for (int j = 1 - (i % 2); j < 8; j += 2) n += gen_loc_moves(s, mkloc(i, j), &result[n], capture);
  return n;
}

/* State::genMoves (state.cu:239-245): captures are forced. */
int or_genmoves(const or_state *s, or_move *result) {
  int n = gen_type_moves(s, result, 1);
  if (n == 0) n = gen_type_moves(s, result, 0);
  return n;
}

/* State::move (state.cu:57-92) */
void or_apply(or_state *s, const or_move *m) {
  for (int i = 0; i < m->jumps; i++) s->board[m->removed[i].r][m->removed[i].c].occupied = 0;
  or_item *to = &s->board[m->to.r][m->to.c];
  const or_item *from = at(s, m->from);
  to->occupied = 1;
  to->type = m->promoted ? OR_KING : from->type;
  to->owner = from->owner;
  s->board[m->from.r][m->from.c].occupied = 0;
  s->turn = next_turn(s->turn);
  if (m->jumps > 0) s->msc = 0; else s->msc++;
}

/* State::isGameOver / getWinner (state.cpp:16-23) */
int or_is_over(const or_state *s) {
  or_move moves[OR_MAX_MOVES];
  return or_genmoves(s, moves) == 0 || s->msc >= OR_DRAW_PLIES;
}
int or_winner(const or_state *s) { return s->msc < OR_DRAW_PLIES ? next_turn(s->turn) : OR_NONE; }

int or_genmoves_b16(const or_board16 *pos, uint32_t n, or_packed_move *out, uint32_t max_moves,
                    uint8_t *counts) {
  int overflow = 0;
  for (uint32_t i = 0; i < n; i++) {
    or_state s;
    or_move mv[OR_MAX_MOVES];
    or_from_board16(&pos[i], &s);
    int k = or_genmoves(&s, mv);
    counts[i] = (uint8_t)(k > 255 ? 255 : k);
    if ((uint32_t)k > max_moves) { overflow = 1; k = (int)max_moves; }
    for (int j = 0; j < k; j++) or_pack_move(&mv[j], &out[(size_t)i * max_moves + j]);
  }
  return overflow ? -1 : 0;
}

int or_apply_packed_b16(or_board16 *pos, const or_packed_move *pm) {
  or_state s;
  or_move mv[OR_MAX_MOVES];
  or_from_board16(pos, &s);
  int k = or_genmoves(&s, mv);
  for (int j = 0; j < k; j++) {
    or_packed_move p;
    or_pack_move(&mv[j], &p);
    if (memcmp(&p, pm, sizeof(p)) == 0) {
      or_apply(&s, &mv[j]);
      or_to_board16(&s, pos);
      return 0;
    }
  }
  return -1;
}

/* ------------------------------------------------------------------ */
/* heuristic (heuristic.cu:7-49; man = 1, king = 4)                     */
/* ------------------------------------------------------------------ */

static inline unsigned piece_value(int type) { return type == OR_KING ? 4u : 1u; }

void or_score_state(const or_state *s, unsigned score[2]) {
  score[0] = score[1] = 0;
  for (int i = 0; i < 8; i++)
    for (int j = 1 - (i % 2); j < 8; j += 2)
      if (s->board[i][j].occupied) score[s->board[i][j].owner] += piece_value(s->board[i][j].type);
}

void or_score_move(const or_state *s, const or_move *m, int score[2]) {
  score[0] = score[1] = 0;
  if (m->promoted) score[s->turn] += 4 - 1;
  for (int i = 0; i < m->jumps; i++)
    score[next_turn(s->turn)] -= (int)piece_value(at(s, m->removed[i])->type);
}

float or_get_weight(const or_state *s, const unsigned ss[2], const int ms[2]) {
  int t = s->turn, o = next_turn(s->turn);
  return (float)(ss[t] + ms[t]) / (ss[o] + ms[o]);
}

/* ------------------------------------------------------------------ */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: */
/* as easy as 1, 2, 3", SC'11)                                          */
/* ------------------------------------------------------------------ */

void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int round = 0; round < 10; round++) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c0 = hi1 ^ c1 ^ k0;
    c1 = lo1;
    c2 = hi0 ^ c3 ^ k1;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

uint32_t or_stream_draw(uint64_t seed, uint64_t id, uint32_t tag, uint32_t k) {
  uint32_t ctr[4] = {k >> 2, (uint32_t)id, (uint32_t)(id >> 32), tag};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t out[4];
  or_philox4x32_10(ctr, key, out);
  return out[k & 3];
}

static inline uint32_t mulhi_idx(uint32_t r, uint32_t n) { return (uint32_t)(((uint64_t)r * n) >> 32); }

/* ------------------------------------------------------------------ */
/* project playout policies, restated over the reference move list      */
/* ------------------------------------------------------------------ */

/* Fixed-point heuristic noise: Irwin-Hall sum of four 16-bit uniforms,
 * centred and scaled to sigma ~= 0.11 in Q16 (HEURISTIC_SIGMA,
 * heuristic.hpp:5). */
#define HEUR_NOISE_K 12486
static inline int32_t heur_noise_q16(uint32_t a, uint32_t b) {
  int32_t sum = (int32_t)(a & 0xffffu) + (int32_t)(a >> 16) + (int32_t)(b & 0xffffu) + (int32_t)(b >> 16);
  int64_t x = (int64_t)(sum - 131070) * HEUR_NOISE_K;
  return (int32_t)(x >> 16);
}

/* getWeight (heuristic.cu:44-49) in Q16: (own + d_own) / (opp + d_opp). */
static inline int32_t heur_weight_q16(int num, int den) {
  if (den <= 0) return 0x3fffffff;
  return (int32_t)(((uint32_t)num << 16) / (uint32_t)den);
}

/* eps-greedy evaluation change of a move for the mover: men 4, kings 8,
 * plus one unit per row a man has advanced (P1 forward = +row). */
static inline int adv_of(int turn, int row) { return turn == OR_P1 ? row : 7 - row; }

static int eps_delta(const or_state *s, const or_move *m) {
  int d = 0;
  const or_item *it = at(s, m->from);
  for (int i = 0; i < m->jumps; i++) {
    const or_item *c = at(s, m->removed[i]);
    if (c->type == OR_KING) d += 8;
    else d += 4 + adv_of(c->owner, m->removed[i].r);
  }
  if (it->type == OR_MAN) {
    if (m->promoted) d += 4 - adv_of(s->turn, m->from.r);
    else d += adv_of(s->turn, m->to.r) - adv_of(s->turn, m->from.r);
  }
  return d;
}

#define EPS_THRESHOLD 429496730u /* ceil(0.1 * 2^32) */

/* choose a move index for one ply; *k counts stream draws */
static int choose(const or_state *s, const or_move *mv, int n, int policy, uint64_t seed, uint64_t id,
                  uint32_t tag, uint32_t *k) {
  if (n < 2) return 0;
  if (policy == 1) {
    unsigned ss[2];
    or_score_state(s, ss);
    int t = s->turn, o = next_turn(s->turn);
    int best = -1;
    int32_t bestw = 0;
    for (int j = 0; j < n; j++) {
      int ms[2];
      or_score_move(s, &mv[j], ms);
      uint32_t a = or_stream_draw(seed, id, tag, (*k)++);
      uint32_t b = or_stream_draw(seed, id, tag, (*k)++);
      int32_t w = heur_weight_q16((int)ss[t] + ms[t], (int)ss[o] + ms[o]) + heur_noise_q16(a, b);
      if (best < 0 || w > bestw) { best = j; bestw = w; }
    }
    return best;
  }
  if (policy == 2) {
    uint32_t r0 = or_stream_draw(seed, id, tag, (*k)++);
    if (r0 < EPS_THRESHOLD) return (int)mulhi_idx(or_stream_draw(seed, id, tag, (*k)++), (uint32_t)n);
    int bestd = -1000000, ties = 0;
    for (int j = 0; j < n; j++) {
      int d = eps_delta(s, &mv[j]);
      if (d > bestd) { bestd = d; ties = 1; } else if (d == bestd) ties++;
    }
    uint32_t pick = 0;
    if (ties > 1) pick = mulhi_idx(or_stream_draw(seed, id, tag, (*k)++), (uint32_t)ties);
    for (int j = 0; j < n; j++)
      if (eps_delta(s, &mv[j]) == bestd) { if (pick == 0) return j; pick--; }
    return 0;
  }
  return (int)mulhi_idx(or_stream_draw(seed, id, tag, (*k)++), (uint32_t)n);
}

int or_replay_playout(const or_board16 *pos, uint64_t seed, uint64_t id, int policy, uint32_t *plies,
                      uint32_t *draws) {
  or_state s;
  or_move mv[OR_MAX_MOVES];
  or_from_board16(pos, &s);
  uint32_t k = 0, p = 0;
  int outcome;
  for (;;) {
    if (s.msc >= OR_DRAW_PLIES) { outcome = 0; break; }
    int n = or_genmoves(&s, mv);
    if (n == 0) { outcome = s.turn == OR_P1 ? -1 : 1; break; }
    int i = choose(&s, mv, n, policy, seed, id, 0, &k);
    or_apply(&s, &mv[i]);
    p++;
  }
  if (plies) *plies = p;
  if (draws) *draws = k;
  return outcome;
}

void or_replay_batch(const or_board16 *pos, const uint32_t *reps, uint32_t npos, uint64_t seed,
                     uint64_t stream_base, int policy, int8_t *out, uint32_t *plies, int nthreads) {
  uint64_t *off = (uint64_t *)malloc(sizeof(uint64_t) * (npos + 1));
  off[0] = 0;
  for (uint32_t p = 0; p < npos; p++) off[p + 1] = off[p] + reps[p];
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
  for (int64_t p = 0; p < (int64_t)npos; p++)
    for (uint64_t j = off[p]; j < off[p + 1]; j++) {
      uint32_t pl = 0;
      out[j] = (int8_t)or_replay_playout(&pos[p], seed, stream_base + j, policy, &pl, NULL);
      if (plies) plies[j] = pl;
    }
  (void)nthreads;
  free(off);
}

void or_random_positions(uint64_t seed, uint32_t n, uint32_t min_plies, uint32_t max_plies,
                         or_board16 *out) {
  for (uint32_t p = 0; p < n; p++) {
    or_state s;
    or_move mv[OR_MAX_MOVES];
    or_start_state(&s);
    uint32_t k = 0;
    uint32_t span = max_plies - min_plies + 1;
    uint32_t np = min_plies + mulhi_idx(or_stream_draw(seed, p, 1, k++), span);
    for (uint32_t ply = 0; ply < np; ply++) {
      if (s.msc >= OR_DRAW_PLIES) break;
      int nm = or_genmoves(&s, mv);
      if (nm == 0) break;
      int i = choose(&s, mv, nm, 0, seed, p, 1, &k);
      or_apply(&s, &mv[i]);
    }
    or_to_board16(&s, &out[p]);
  }
}

/* ------------------------------------------------------------------ */
/* reference host drivers restated (CPU baseline, kind "port")          */
/* ------------------------------------------------------------------ */

/* State::getMoves (state.cpp:10-14) returns a heap-allocated vector. */
static or_move *get_moves(const or_state *s, int *n) {
  or_move tmp[OR_MAX_MOVES];
  *n = or_genmoves(s, tmp);
  or_move *v = (or_move *)malloc(sizeof(or_move) * (size_t)(*n > 0 ? *n : 1));
  memcpy(v, tmp, sizeof(or_move) * (size_t)*n);
  return v;
}

/* HostPlayoutDriver::runPlayouts (playout.cpp:17-32) with
 * RandomPlayer::getMove (player.cpp:13-16): isGameOver() and getMove() each
 * generate the move list, and the move is rand() % n. */
void or_host_playouts(const or_board16 *states, uint32_t n, int8_t *out, int nthreads,
                      unsigned srand_seed) {
  srand(srand_seed);
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for num_threads(nthreads)
#endif
  for (int64_t i = 0; i < (int64_t)n; i++) {
    or_state s;
    or_from_board16(&states[i], &s);
    for (;;) {
      int k;
      or_move *v = get_moves(&s, &k);
      free(v);
      if (k == 0 || s.msc >= OR_DRAW_PLIES) break;
      v = get_moves(&s, &k);
      or_move m = v[rand() % k];
      free(v);
      or_apply(&s, &m);
    }
    int w = or_winner(&s);
    out[i] = (int8_t)(w == OR_P1 ? 1 : (w == OR_P2 ? -1 : 0));
  }
  (void)nthreads;
}

/* The noise source of HostHeuristicPlayoutDriver (heuristicPlayout.cpp:14-15):
 * one std::default_random_engine (minstd_rand0: x = 16807 x mod 2^31 - 1) and
 * one normal_distribution, shared by every OpenMP thread.  The reference
 * shares them unsynchronised; here the shared words are read and written with
 * relaxed atomic loads and stores, so the threads contend for the same cache
 * lines without a data race (concurrent callers may repeat a draw, as they
 * can in the reference).  N(0, sigma) by the polar method, the second deviate
 * kept for the next call. */
static _Atomic uint64_t g_engine = 1;
static _Atomic int g_have_saved = 0;
static _Atomic double g_saved = 0.0;

static double engine_uniform(void) {
  uint64_t x = atomic_load_explicit(&g_engine, memory_order_relaxed);
  x = (x * 16807u) % 2147483647u;
  atomic_store_explicit(&g_engine, x, memory_order_relaxed);
  return (double)(x - 1) / 2147483646.0;
}

static float shared_normal(float sigma) {
  if (atomic_load_explicit(&g_have_saved, memory_order_relaxed)) {
    atomic_store_explicit(&g_have_saved, 0, memory_order_relaxed);
    return (float)(atomic_load_explicit(&g_saved, memory_order_relaxed) * sigma);
  }
  for (;;) {
    const double u = 2.0 * engine_uniform() - 1.0, v = 2.0 * engine_uniform() - 1.0;
    const double q = u * u + v * v;
    if (q > 0.0 && q < 1.0) {
      const double f = sqrt(-2.0 * log(q) / q);
      atomic_store_explicit(&g_saved, u * f, memory_order_relaxed);
      atomic_store_explicit(&g_have_saved, 1, memory_order_relaxed);
      return (float)(v * f * sigma);
    }
  }
}

/* HostHeuristicPlayoutDriver::runPlayouts (heuristicPlayout.cpp:12-48):
 * isGameOver() and getMoves() each generate the move list, every move is
 * scored and weighted, and the noise comes from the shared engine above,
 * restarted for each call (the reference constructs it per call). */
void or_host_heuristic_playouts(const or_board16 *states, uint32_t n, int8_t *out, uint64_t seed) {
  atomic_store(&g_engine, (uint64_t)(seed % 2147483646u) + 1u);
  atomic_store(&g_have_saved, 0);
#ifdef _OPENMP
#pragma omp parallel for
#endif
  for (int64_t i = 0; i < (int64_t)n; i++) {
    or_state s;
    or_from_board16(&states[i], &s);
    unsigned ss[2];
    or_score_state(&s, ss);
    for (;;) {
      int k;
      or_move *v = get_moves(&s, &k);
      free(v);
      if (k == 0 || s.msc >= OR_DRAW_PLIES) break;
      v = get_moves(&s, &k);
      int best = -1, bms[2] = {0, 0};
      float bw = -INFINITY;
      for (int j = 0; j < k; j++) {
        int ms[2];
        or_score_move(&s, &v[j], ms);
        float w = or_get_weight(&s, ss, ms) + shared_normal(0.11f);
        if (w > bw) { best = j; bw = w; bms[0] = ms[0]; bms[1] = ms[1]; }
      }
      or_apply(&s, &v[best]);
      free(v);
      ss[0] += bms[0]; ss[1] += bms[1];
    }
    int w = or_winner(&s);
    out[i] = (int8_t)(w == OR_P1 ? 1 : (w == OR_P2 ? -1 : 0));
  }
}
