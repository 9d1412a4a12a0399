"""CPU restatement of the device-resident searches (test infrastructure only).

Restates, step by step, what one step of gpu_ai_gb300/csrc/search.cu does to
every search's tree, so that a GPU test can compare the trees node for node:

  quota      leaf slots per search: min(Q, ceil(remaining budget / playouts
             per leaf)), searches in slot order;
  select     the level-synchronous split of the reference's GameTree::select
             (src/mcts.cpp:63-157): a terminal node or an unexpanded node with
             one slot is a leaf; an unexpanded node with more slots is expanded
             (its children in move-list order) and its slots are split: untried
             children share them equally, otherwise in proportion to UCB1
             weights rounded down, the rest one each to the heaviest children
             (first on ties).  The frontier is handled in chunks of 32 entries
             (one warp's lanes; on steps of 128 leaves per search or more a
             block of 128, 256 or 512 threads); a chunk's expansions take node indices in
             entry order, and an expansion whose inclusive prefix of children
             would pass the search's node range plays out instead;
  playouts   slot i of a search's step uses random streams stream_next + i * ppl
             onward; the outcomes come from the caller (the oracle's replay of
             the playout kernel);
  backprop   every node on a leaf's path gets its playouts and, in half points,
             the score of the player who moved into it (GameTree::update,
             src/mcts.cpp:159-180).

Learned searches (a network attached) restate leaf_eval_kernel (tanh value,
priors = softmax of the legal moves' logits, a (from, to) pair's share split
equally among the moves that have it), split_puct (PUCT with virtual visits,
first-play urgency = parent's mean - 0.1) and backprop_learned_kernel (64
visit units per slot, leaf result = w * network value + (1 - w) * playout
mean).  The network's outputs are supplied by the caller per leaf slot.

Arithmetic: "device" mode does every float operation in float32 in the
kernels' order with the kernels' own elementary functions (detmath.cuh:
det_log, det_exp, det_tanh), so results are bit-identical; "reference" mode
is GameTree's double arithmetic with its child-to-move perspective and wins
only (src/mcts.cpp:183-191), which pins the split and update structure to the
reference's own tree on CPU.

Move generation and playouts are injected: children(board) -> (boards,
moves) in move-list order, playouts(boards, reps, seed, stream_base, policy)
-> int8 outcomes.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Callable, List, Optional

import numpy as np

F = np.float32
EXPANDED, TERMINAL, EVALUATED = 1, 2, 4
DRAW_PLIES = 50
MAX_CHILDREN = 64
UNITS = 64
PRIORS = 32
TERMINAL_LEAF = F(2.0)
def select_team(Q: int) -> int:
    """Frontier entries per round of select_kernel for a step of Q leaves per
    search: a warp (32) below 128, else a block of 128, 256 or 512 threads."""
    return 32 if Q < 128 else (128 if Q < 256 else (256 if Q < 512 else 512))


def _cf(bits: int) -> np.float32:
    return np.array(bits, np.uint32).view(np.float32)[()]


LN2, LOG2E, LN2_HI, LN2_LO = _cf(0x3f317218), _cf(0x3fb8aa3b), _cf(0x3f317200), _cf(0x35bfbe8e)
SQRT2 = _cf(0x3fb504f3)
INV_ODD = [_cf(0x3dba2e8c), _cf(0x3de38e39), _cf(0x3e124925), _cf(0x3e4ccccd), _cf(0x3eaaaaab)]  # 1/11 .. 1/3
INV_FACT = [_cf(0x39500d01), _cf(0x3ab60b61), _cf(0x3c088889), _cf(0x3d2aaaab), _cf(0x3e2aaaab)]  # 1/7! .. 1/3!
UCB_C = F(1.41421356)
FPU_REDUCTION = F(0.1)


def det_log(x) -> np.float32:
    """det_log of detmath.cuh: x = m 2^e, ln m = 2 atanh((m-1)/(m+1)) by its series to s^11."""
    u = int(np.array(F(x)).view(np.uint32))
    e = (u >> 23) - 127
    m = _cf((u & 0x7FFFFF) | 0x3F800000)
    if m > SQRT2:
        m = m * F(0.5)
        e += 1
    s = (m - F(1)) / (m + F(1))
    s2 = s * s
    p = INV_ODD[0]
    for c in INV_ODD[1:]:
        p = p * s2 + c
    p = p * s2 + F(1)
    return F(e) * LN2 + (F(2) * s) * p


def det_exp(x) -> np.float32:
    """det_exp of detmath.cuh for x <= 0: Cody-Waite reduction, degree-7 Taylor polynomial."""
    x = F(x)
    if not (x >= F(-87.0)):
        return F(0)
    k = np.rint(x * LOG2E)
    r = (x - k * LN2_HI) - k * LN2_LO
    p = INV_FACT[0]
    for c in INV_FACT[1:]:
        p = p * r + c
    p = p * r + F(0.5)
    p = p * r + F(1)
    p = p * r + F(1)
    return p * _cf((int(k) + 127) << 23)


def det_tanh(x) -> np.float32:
    x = F(x)
    a = abs(x)
    if a > F(9):
        y = F(1)
    else:
        t = det_exp(F(-2) * a)
        y = (F(1) - t) / (F(1) + t)
    return -y if x < F(0) else y


@dataclass
class Node:
    board: tuple
    parent: int
    first: int = -1
    k: int = 0
    state: int = 0
    visits: int = 0
    score2: int = 0
    wins: list = field(default_factory=lambda: [0, 0])  # reference mode: wins of PLAYER_1, PLAYER_2
    priors: Optional[np.ndarray] = None  # float16 x PRIORS


@dataclass
class Search:
    root_board: tuple
    budget: int
    cap: int
    stream_next: int
    nodes: List[Node] = field(default_factory=list)
    done: int = 0


def side_to_move(board) -> int:
    return int(board[3]) & 1


class SearchesOracle:
    def __init__(self, max_searches: int, playouts_per_leaf: int, policy: int, seed: int,
                 children: Callable, playouts: Optional[Callable] = None, mode: str = "device",
                 learned: Optional[dict] = None):
        self.slots: List[Optional[Search]] = [None] * max_searches
        self.ppl = playouts_per_leaf
        self.policy = policy
        self.seed = seed
        self.children = children
        self.playouts = playouts
        self.mode = mode
        self.learned = learned  # {"value_weight": w, "c_puct": c} or None
        self.last_leaves = []

    # ------------------------------------------------------------------ searches

    def add(self, root, budget: int, node_capacity: int, stream_base: int) -> int:
        slot = next(i for i, s in enumerate(self.slots) if s is None)
        board = tuple(int(v) for v in root)
        s = Search(board, budget, node_capacity, stream_base)
        s.nodes.append(Node(board, -1, state=TERMINAL if self._over(board) else 0))
        self.slots[slot] = s
        return slot

    def remove(self, slot: int):
        self.slots[slot] = None

    def _over(self, board) -> bool:
        if (int(board[3]) >> 8) & 0xFF >= DRAW_PLIES:
            return True
        return len(self.children(board)[0]) == 0

    def child_count(self, board) -> int:
        """child_count of search.cu: legal moves, 0 for a finished game or more than 64 moves."""
        if (int(board[3]) >> 8) & 0xFF >= DRAW_PLIES:
            return 0
        k = len(self.children(board)[0])
        return k if 0 < k <= MAX_CHILDREN else 0

    def _expand(self, s: Search, n: int, first: int, k: int):
        boards, _ = self.children(s.nodes[n].board)
        assert len(boards) == k
        assert len(s.nodes) == first, "expansions take consecutive node indices"
        for b in boards:
            s.nodes.append(Node(tuple(int(v) for v in b), n))
        nd = s.nodes[n]
        nd.first, nd.k = first, k
        nd.state |= EXPANDED

    # ------------------------------------------------------------------ splits

    def _ucb_device(self, c: Node, lnN):
        mean = (F(0.5) * F(c.score2)) / F(c.visits)
        return mean + UCB_C * np.sqrt(lnN / F(c.visits), dtype=np.float32)

    def _split_device(self, s: Search, nd: Node, first: int, k: int, T: int):
        """split_slots of search.cu in float32."""
        kids = [s.nodes[first + c] for c in range(k)]
        lnN = det_log(F(nd.visits if nd.visits > 0 else 1))
        wsum = F(0)
        untried = 0
        for c in kids:
            if c.visits == 0:
                untried += 1
            else:
                wsum = wsum + self._ucb_device(c, lnN)
        equal = untried == 0 and not (wsum > F(0))
        w, give = [], []
        for c in kids:
            wc = F(3.0e38) if c.visits == 0 else (F(1) if equal else self._ucb_device(c, lnN))
            w.append(wc)
            if untried > 0:
                give.append(T // untried if c.visits == 0 else 0)
            else:
                give.append(int(F(T) * (wc / (F(k) if equal else wsum))))
        self._remainder(w, give, T, F(-1))
        return give

    def _split_reference(self, s: Search, nd: Node, first: int, k: int, T: int):
        """GameTree::select's split (src/mcts.cpp:94-136) in double, ucb1 of src/mcts.cpp:183-191."""
        kids = [s.nodes[first + c] for c in range(k)]
        lp = math.log(float(nd.visits)) if nd.visits else 0.0
        w = []
        for c in kids:
            if c.visits == 0:
                w.append(math.inf)
            else:
                turn = side_to_move(c.board)
                e = np.sqrt(np.longdouble(2) * np.longdouble(lp) / np.longdouble(c.visits))
                w.append(float(np.longdouble(float(c.wins[turn]) / float(c.visits)) + e))
        wsum = 0.0
        for x in w:
            wsum += x
        untried = sum(1 for c in kids if c.visits == 0)
        give = []
        for i, c in enumerate(kids):
            if untried > 0:
                give.append(T // untried if c.visits == 0 else 0)
            else:
                give.append(int(T * (w[i] / wsum)))
        self._remainder(w, give, T, -math.inf)
        return give

    @staticmethod
    def _remainder(w, give, T, lowest):
        taken = [False] * len(w)
        assigned = sum(give)
        while assigned < T:
            mw, opt = lowest, -1
            for c in range(len(w)):
                if not taken[c] and w[c] > mw:
                    mw, opt = w[c], c
            assert opt >= 0
            taken[opt] = True
            give[opt] += 1
            assigned += 1

    def _split_puct(self, s: Search, nd: Node, first: int, k: int, T: int):
        """split_puct of search.cu in float32."""
        c_puct = F(self.learned["c_puct"])
        kids = [s.nodes[first + c] for c in range(k)]
        priors = bool(nd.state & EVALUATED) and k <= PRIORS
        if nd.visits:
            fpu = max(F(0), (F(1) - (F(0.5) * F(nd.score2)) / F(nd.visits)) - FPU_REDUCTION)
        else:
            fpu = F(0.5)
        uniform = F(1) / F(k)
        q, nv, pr, u = [], [], [], []
        for i, c in enumerate(kids):
            q.append((F(0.5) * F(c.score2)) / F(c.visits) if c.visits else fpu)
            nv.append(F(1) + F(c.visits // UNITS))
            pr.append(c_puct * (F(nd.priors[i]) if priors else uniform))
            u.append(pr[-1] / nv[-1])
        give = [0] * k
        N = F(nd.visits // UNITS)
        for t in range(T):
            sq = np.sqrt((N + F(t)) + F(1), dtype=np.float32)
            best, bs = 0, F(-3.0e38)
            for c in range(k):
                sc = sq * u[c] + q[c]
                if sc > bs:
                    bs, best = sc, c
            give[best] += 1
            nv[best] = nv[best] + F(1)
            u[best] = pr[best] / nv[best]
        return give

    # ------------------------------------------------------------------ one step

    def quota(self, Q: int):
        qs = []
        for s in self.slots:
            q = 0
            if s is not None and s.done < s.budget:
                need = (s.budget - s.done + self.ppl - 1) // self.ppl
                q = min(need, Q)
            qs.append(q)
        return qs

    def select(self, s: Search, q: int, team: int = 32):
        """select_kernel for one search: list of leaf node indices in emission
        order.  `team`: frontier entries handled per round (select_team)."""
        learned = self.learned is not None
        leaves = []
        frontier = [(0, q)]
        while frontier:
            nxt = []
            for base in range(0, len(frontier), team):
                chunk = frontier[base:base + team]
                ent = []
                for n, T in chunk:
                    nd = s.nodes[n]
                    leaf, grow = 0, 0
                    if nd.state & TERMINAL:
                        leaf = T
                    elif not nd.state & EXPANDED:
                        if learned:
                            if nd.state & EVALUATED:
                                grow = self.child_count(nd.board)
                            if grow == 0:
                                leaf = T
                        else:
                            if T == 1:
                                leaf = 1
                            else:
                                grow = self.child_count(nd.board)
                            if T > 1 and grow == 0:
                                leaf = T
                    ent.append([n, T, leaf, grow, nd.first, nd.k])
                gx, fit_end = 0, 0
                node_next = len(s.nodes)
                for e in ent:
                    gx += e[3]
                    if e[3] > 0 and node_next + gx <= s.cap:
                        e[4], e[5] = node_next + gx - e[3], e[3]
                        self._expand(s, e[0], e[4], e[5])
                        fit_end = gx
                    elif e[3] > 0:
                        e[2] = e[1]
                for n, T, leaf, grow, first, k in ent:
                    if leaf:
                        leaves.extend([n] * leaf)
                        continue
                    nd = s.nodes[n]
                    if learned:
                        give = self._split_puct(s, nd, first, k, T)
                    elif self.mode == "device":
                        give = self._split_device(s, nd, first, k, T)
                    else:
                        give = self._split_reference(s, nd, first, k, T)
                    nxt.extend((first + c, g) for c, g in enumerate(give) if g)
            frontier = nxt
        return leaves

    def step(self, Q: int, net_value=None, net_logits=None, outcomes=None):
        """One step over all searches.  Returns the leaf slots [(slot, node,
        board, first stream id, outcomes)] in the device's slot order.  For
        learned searches net_value / net_logits hold the network's raw value
        and float32 logits per leaf slot, in that order.  `outcomes` (slots x
        playouts per leaf), when given, stands in for the replayed playouts
        (learned-proposal playouts, whose parity is checked on their own)."""
        qs = self.quota(Q)
        team = select_team(Q)
        slots = []
        for si, (s, q) in enumerate(zip(self.slots, qs)):
            if s is None or q == 0:
                continue
            leaves = self.select(s, q, team)
            assert len(leaves) == q
            for i, n in enumerate(leaves):
                slots.append([si, n, s.nodes[n].board, s.stream_next + i * self.ppl, None])
            s.stream_next += q * self.ppl
        if outcomes is None:
            self._playouts(slots)
        else:
            assert len(outcomes) == len(slots)
            for sl, o in zip(slots, outcomes):
                sl[4] = np.asarray(o, np.int8)
        if self.learned is not None:
            values = self._leaf_eval(slots, net_value, net_logits)
            self._backprop_learned(slots, values)
        else:
            self._backprop(slots)
        self.last_leaves = slots
        return slots

    def _playouts(self, slots):
        if not slots:
            return
        # each search's slots use consecutive stream ids: one replay call per search
        i = 0
        while i < len(slots):
            j = i
            while j < len(slots) and slots[j][0] == slots[i][0]:
                j += 1
            boards = np.array([sl[2] for sl in slots[i:j]], np.uint32)
            reps = np.full(j - i, self.ppl, np.uint32)
            out = self.playouts(boards, reps, self.seed, slots[i][3], self.policy)
            for k in range(i, j):
                slots[k][4] = np.asarray(out[(k - i) * self.ppl:(k - i + 1) * self.ppl], np.int8)
            i = j

    def _path(self, s: Search, n: int):
        while n >= 0:
            yield s.nodes[n]
            n = s.nodes[n].parent

    def _backprop(self, slots):
        for si, n, board, _, out in slots:
            s = self.slots[si]
            w1, w2 = int((out > 0).sum()), int((out < 0).sum())
            dr = self.ppl - w1 - w2
            for nd in self._path(s, n):
                mover = side_to_move(nd.board) ^ 1
                nd.visits += self.ppl
                nd.score2 += 2 * (w1 if mover == 0 else w2) + dr
                nd.wins[0] += w1
                nd.wins[1] += w2
            s.done += self.ppl

    def _leaf_eval(self, slots, net_value, net_logits):
        values = []
        for i, (si, n, board, _, _) in enumerate(slots):
            s = self.slots[si]
            boards, moves = self.children(board)
            k = len(boards)
            over = k == 0 or (int(board[3]) >> 8) & 0xFF >= DRAW_PLIES
            values.append(TERMINAL_LEAF if over else det_tanh(net_value[i]))
            nd = s.nodes[n]
            if over or nd.state & (EVALUATED | TERMINAL):
                continue
            if 1 <= k <= PRIORS:
                pairs, of, mult = [], [], []
                for m in moves:
                    pi = int(m[0]) * 32 + int(m[1])
                    if pi not in pairs:
                        pairs.append(pi)
                        mult.append(0)
                    u = pairs.index(pi)
                    mult[u] += 1
                    of.append(u)
                lg = [F(net_logits[i][p]) for p in pairs]
                lmax = max(lg)
                tot = F(0)
                for x in lg:
                    tot = tot + det_exp(x - lmax)
                pri = np.zeros(PRIORS, np.float16)
                for j in range(k):
                    u = of[j]
                    pri[j] = np.float16((det_exp(lg[u] - lmax) / tot) / F(mult[u]))
                nd.priors = pri
            nd.state |= EVALUATED
        return values

    def _backprop_learned(self, slots, values):
        vw = F(self.learned["value_weight"])
        for (si, n, board, _, out), v in zip(slots, values):
            s = self.slots[si]
            pm = F(int(out.astype(np.int64).sum())) / F(self.ppl)
            x1 = pm
            if v <= F(1):
                v1 = -v if side_to_move(board) else v
                x1 = vw * v1 + (F(1) - vw) * pm
            x1 = min(F(1), max(F(-1), x1))
            s1 = int(np.rint(F(UNITS) * (F(1) + x1)))
            s2 = 2 * UNITS - s1
            for nd in self._path(s, n):
                mover = side_to_move(nd.board) ^ 1
                nd.visits += UNITS
                nd.score2 += s1 if mover == 0 else s2
            s.done += self.ppl

    # ------------------------------------------------------------------ views

    def tree(self, slot: int):
        """info (n, 4) / boards (n, 4) / parent (n,) as gpuai_searches_nodes reports them."""
        s = self.slots[slot]
        info = np.zeros((len(s.nodes), 4), np.uint32)
        boards = np.zeros((len(s.nodes), 4), np.uint32)
        parent = np.zeros(len(s.nodes), np.int32)
        for i, nd in enumerate(s.nodes):
            info[i] = [0xFFFFFFFF if nd.first < 0 else nd.first, nd.k | (nd.state << 16), nd.visits, nd.score2]
            boards[i] = nd.board
            parent[i] = nd.parent
        return {"info": info, "boards": boards, "parent": parent}

    def priors(self, slot: int) -> np.ndarray:
        s = self.slots[slot]
        out = np.zeros((len(s.nodes), PRIORS), np.float16)
        for i, nd in enumerate(s.nodes):
            if nd.priors is not None:
                out[i] = nd.priors
        return out

    def root_stats(self, slot: int):
        """Per root child [playouts, wins of PLAYER_1, wins of PLAYER_2] (wins 0 for
        finished games), as the reference tree runner reports them."""
        s = self.slots[slot]
        r = s.nodes[0]
        rows = []
        for c in range(r.k):
            nd = s.nodes[r.first + c]
            stats = nd.visits > 0 and not self._over(nd.board)
            rows.append([nd.visits, nd.wins[0] if stats else 0, nd.wins[1] if stats else 0])
        return np.array(rows, np.uint32).reshape(-1, 3)
