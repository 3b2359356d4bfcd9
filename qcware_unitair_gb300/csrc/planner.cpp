// Host-side circuit planner: gate list -> fused stages, register layouts,
// gate records and the matrix pool, ready for one transfer to the device.
//
// It follows the same rules as the Python reference implementation in
// fusion.py (plan, _plan_layouts, _record, _layout_record); a CPU test
// checks that both produce identical bytes.  Stages: greedy in circuit
// order, each owning m tile bits of which the lowest c_min are always
// present; a gate needs its dense target bits (a controlled-U only its
// target, a diagonal nothing).  Layouts: greedy groups of a stage's gates
// whose register-needing bits fit rb register bits.
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <complex>
#include <vector>

#include "gbsv.h"

namespace {

using cd = std::complex<double>;

enum { K_DENSE = 0, K_DIAG = 1, K_CTRL = 2 };
enum {
  FG_DENSE1 = 0, FG_DENSE2 = 1, FG_DIAG = 2, FG_CDENSE1 = 3, FG_REAL1 = 4,
  FG_ANTI1 = 5, FG_CANTI1 = 6, FG_PERM2 = 7, FG_RDIAG = 8
};

struct Ctx {
  const gbsv_gate_desc_t* g;
  const cd* mats;
  int n, m, c_min, rb;
};

int pos_of(const Ctx& c, int q) { return c.n - 1 - q; }

// element (r, col) of batch entry b of gate gi's d x d matrix
cd el(const Ctx& c, int gi, int b, int r, int col) {
  const gbsv_gate_desc_t& d = c.g[gi];
  const int dim = 1 << d.nq;
  return c.mats[d.mat + (int64_t)b * d.mat_bstride + r * dim + col];
}

int batch_of(const gbsv_gate_desc_t& d) {
  return d.mat_bstride > 0 ? (int)d.num_batch : 1;
}

// 2x2 block (r0.., c0..) predicates over every batch entry
bool all_b(const Ctx& c, int gi, bool (*pred)(const Ctx&, int, int, int),
           int off) {
  for (int b = 0; b < batch_of(c.g[gi]); ++b)
    if (!pred(c, gi, b, off)) return false;
  return true;
}
bool anti_p(const Ctx& c, int gi, int b, int o) {
  return el(c, gi, b, o, o) == cd(0) && el(c, gi, b, o + 1, o + 1) == cd(0);
}
bool unit_p(const Ctx& c, int gi, int b, int o) {
  return el(c, gi, b, o, o + 1) == cd(1) && el(c, gi, b, o + 1, o) == cd(1);
}
bool real_p(const Ctx& c, int gi, int b, int o) {
  for (int r = 0; r < 2; ++r)
    for (int k = 0; k < 2; ++k)
      if (el(c, gi, b, o + r, o + k).imag() != 0) return false;
  return true;
}

// kind and flag for a 2x2 (offset o = 0 for a 1-qubit gate, 2 for the U
// block of a controlled gate)
void dense1_kind(const Ctx& c, int gi, int o, int* kind, int* flag) {
  if (all_b(c, gi, anti_p, o)) {
    *kind = FG_ANTI1;
    *flag = all_b(c, gi, unit_p, o) ? 1 : 0;
  } else if (all_b(c, gi, real_p, o)) {
    *kind = FG_REAL1;
    *flag = 0;
  } else {
    *kind = FG_DENSE1;
    *flag = 0;
  }
}

int perm_code(const Ctx& c, int gi) {
  const int B = batch_of(c.g[gi]);
  int code = 0;
  for (int r = 0; r < 4; ++r) {
    int src = -1;
    for (int col = 0; col < 4; ++col) {
      bool one = true, zero = true;
      for (int b = 0; b < B; ++b) {
        const cd v = el(c, gi, b, r, col);
        if (v != cd(1)) one = false;
        if (v != cd(0)) zero = false;
        if (v != cd(0) && v != cd(1)) return -1;
      }
      if (one) {
        if (src >= 0) return -1;
        src = col;
      } else if (!zero) {
        return -1;
      }
    }
    if (src < 0) return -1;
    code |= src << (2 * r);
  }
  return code;
}

// needed tile bits (positions) of a gate, or -1 when it cannot be staged
int64_t needs(const Ctx& c, int gi) {
  const gbsv_gate_desc_t& d = c.g[gi];
  if (d.nq > 2) return -1;
  const int p0 = pos_of(c, d.q0);
  const int p1 = d.nq == 2 ? pos_of(c, d.q1) : 0;
  if (d.kind == K_DIAG) return 0;
  if (d.kind == K_CTRL && d.nq == 2) return int64_t(1) << p1;
  int64_t s = int64_t(1) << p0;
  if (d.nq == 2) s |= int64_t(1) << p1;
  return s;
}

int popc(uint64_t x) { return __builtin_popcountll(x); }

struct Out {
  gbsv_plan_t* p;
  int num_ops = 0, num_records = 0, num_layouts = 0;
  int64_t pool_len = 0;
  bool overflow = false;
};

gbsv_fused_gate_t* new_record(Out& o) {
  if (o.num_records >= o.p->max_records) {
    o.overflow = true;
    return nullptr;
  }
  gbsv_fused_gate_t* r = &o.p->records[o.num_records++];
  memset(r, 0, sizeof(*r));
  return r;
}

// append the values of gate gi (rows r0.., cols c0.., diagonal or block)
// for every batch entry; returns (offset, bstride)
void add_pool(Out& o, const Ctx& c, int gi, int which, int nvals,
              gbsv_fused_gate_t* rec) {
  const gbsv_gate_desc_t& d = c.g[gi];
  const int B = batch_of(d);
  const int dim = 1 << d.nq;
  if (o.pool_len + (int64_t)B * nvals > o.p->max_pool) {
    o.overflow = true;
    return;
  }
  rec->mat = o.pool_len;
  rec->mat_bstride = d.mat_bstride > 0 ? nvals : 0;
  for (int b = 0; b < B; ++b) {
    for (int k = 0; k < nvals; ++k) {
      cd v;
      if (which == 0) {  // whole matrix, row-major
        v = el(c, gi, b, k / dim, k % dim);
      } else if (which == 1) {  // diagonal
        v = el(c, gi, b, k, k);
      } else {  // lower-right 2x2 block of a 4x4
        v = el(c, gi, b, 2 + k / 2, 2 + k % 2);
      }
      const int64_t at = o.pool_len + (int64_t)b * nvals + k;
      if (o.p->dtype == GBSV_C64) {
        static_cast<float*>(o.p->pool)[2 * at] = (float)v.real();
        static_cast<float*>(o.p->pool)[2 * at + 1] = (float)v.imag();
      } else {
        static_cast<double*>(o.p->pool)[2 * at] = v.real();
        static_cast<double*>(o.p->pool)[2 * at + 1] = v.imag();
      }
    }
  }
  o.pool_len += (int64_t)B * nvals;
}

// gate record for a shared-memory stage (tile bits = local indices)
void plain_record(Out& o, const Ctx& c, int gi, const int* local) {
  const gbsv_gate_desc_t& d = c.g[gi];
  gbsv_fused_gate_t* r = new_record(o);
  if (!r) return;
  const int p0 = pos_of(c, d.q0);
  const int p1 = d.nq == 2 ? pos_of(c, d.q1) : 0;
  if (d.kind == K_DIAG) {
    r->kind = FG_DIAG;
    r->nq = d.nq;
    r->b0 = local[p0] >= 0 ? local[p0] : -1 - p0;
    r->b1 = d.nq == 2 ? (local[p1] >= 0 ? local[p1] : -1 - p1) : 0;
    add_pool(o, c, gi, 1, 1 << d.nq, r);
  } else if (d.kind == K_CTRL && local[p0] < 0) {
    r->kind = FG_DENSE1;
    r->b0 = local[p1];
    r->cmask = r->cval = uint64_t(1) << p0;
    add_pool(o, c, gi, 2, 4, r);
  } else if (d.nq == 1) {
    r->kind = FG_DENSE1;
    r->b0 = local[p0];
    add_pool(o, c, gi, 0, 4, r);
  } else {
    r->kind = FG_DENSE2;
    r->b0 = local[p0];
    r->b1 = local[p1];
    add_pool(o, c, gi, 0, 16, r);
  }
}

// gate record for a register-blocked stage; kreg[tile bit] = register bit
void layout_record(Out& o, const Ctx& c, int gi, const int* local,
                   const int* kreg) {
  const gbsv_gate_desc_t& d = c.g[gi];
  gbsv_fused_gate_t* r = new_record(o);
  if (!r) return;
  const int p0 = pos_of(c, d.q0);
  const int p1 = d.nq == 2 ? pos_of(c, d.q1) : 0;
  auto enc = [&](int p) {
    if (local[p] < 0) return -1 - p;
    if (kreg[local[p]] >= 0) return kreg[local[p]];
    return c.rb + local[p];
  };
  if (d.kind == K_DIAG) {
    r->kind = FG_RDIAG;
    r->nq = d.nq;
    r->b0 = enc(p0);
    r->b1 = d.nq == 2 ? enc(p1) : 0;
    add_pool(o, c, gi, 1, 1 << d.nq, r);
    return;
  }
  if (d.kind == K_CTRL && d.nq == 2) {
    const int t = local[p1];
    if (local[p0] < 0) {
      int kind, flag;
      dense1_kind(c, gi, 2, &kind, &flag);
      r->kind = kind;
      r->nq = flag;
      r->b0 = kreg[t];
      r->cmask = r->cval = uint64_t(1) << p0;
      add_pool(o, c, gi, 2, 4, r);
      return;
    }
    if (kreg[local[p0]] < 0) {
      if (all_b(c, gi, anti_p, 2)) {
        r->kind = FG_CANTI1;
        r->nq = all_b(c, gi, unit_p, 2) ? 1 : 0;
      } else {
        r->kind = FG_CDENSE1;
      }
      r->b0 = kreg[t];
      r->b1 = local[p0];
      add_pool(o, c, gi, 2, 4, r);
      return;
    }
  }
  if (d.nq == 1) {
    int kind, flag;
    dense1_kind(c, gi, 0, &kind, &flag);
    r->kind = kind;
    r->nq = flag;
    r->b0 = kreg[local[p0]];
    add_pool(o, c, gi, 0, 4, r);
    return;
  }
  const int code = perm_code(c, gi);
  r->b0 = kreg[local[p0]];
  r->b1 = kreg[local[p1]];
  if (code >= 0) {
    r->kind = FG_PERM2;
    r->nq = code;
  } else {
    r->kind = FG_DENSE2;
  }
  add_pool(o, c, gi, 0, 16, r);
}

void emit_stage(Out& o, const Ctx& c, uint64_t tile,
                const std::vector<int>& gates, bool layouts) {
  // top up to m bits with the lowest free positions
  for (int p = 0; popc(tile) < c.m; ++p) tile |= uint64_t(1) << p;
  int cc = 0;
  while ((tile >> cc) & 1) ++cc;
  cc = std::min(cc, c.m);
  int order[64], local[64];
  int no = 0;
  for (int p = 0; p < cc; ++p) order[no++] = p;
  for (int p = cc; p < c.n; ++p)
    if ((tile >> p) & 1) order[no++] = p;
  for (int p = 0; p < 64; ++p) local[p] = -1;
  for (int i = 0; i < no; ++i) local[order[i]] = i;
  if (o.num_ops >= o.p->max_ops) {
    o.overflow = true;
    return;
  }
  gbsv_plan_op_t* op = &o.p->ops[o.num_ops++];
  memset(op, 0, sizeof(*op));
  op->contiguous = cc;
  for (int i = 0; i < c.m; ++i) op->positions[i] = order[i];
  if (!layouts) {
    op->type = 1;
    op->first = o.num_records;
    for (int gi : gates) plain_record(o, c, gi, local);
    op->count = o.num_records - op->first;
    return;
  }
  op->type = 2;
  op->first = o.num_layouts;
  // group into register layouts
  std::vector<std::pair<uint64_t, std::vector<int>>> groups;
  uint64_t need_all = 0;
  std::vector<int> cur;
  for (int gi : gates) {
    const gbsv_gate_desc_t& d = c.g[gi];
    uint64_t need = 0;
    if (d.kind == K_DIAG) {
      need = 0;
    } else if (d.kind == K_CTRL && d.nq == 2) {
      need = uint64_t(1) << local[pos_of(c, d.q1)];
    } else {
      need = uint64_t(1) << local[pos_of(c, d.q0)];
      if (d.nq == 2) need |= uint64_t(1) << local[pos_of(c, d.q1)];
    }
    if (popc(need_all | need) <= c.rb) {
      need_all |= need;
      cur.push_back(gi);
    } else {
      groups.emplace_back(need_all, cur);
      need_all = need;
      cur.assign(1, gi);
    }
  }
  groups.emplace_back(need_all, cur);
  for (auto& grp : groups) {
    if (o.num_layouts >= o.p->max_layouts) {
      o.overflow = true;
      return;
    }
    int bits[8], nb = 0;
    for (int b = 0; b < c.m; ++b)
      if ((grp.first >> b) & 1) bits[nb++] = b;
    for (int b = c.m - 1; nb < c.rb; --b)
      if (!((grp.first >> b) & 1)) bits[nb++] = b;
    int kreg[64];
    for (int i = 0; i < 64; ++i) kreg[i] = -1;
    for (int k = 0; k < c.rb; ++k) kreg[bits[k]] = k;
    gbsv_layout_t* L = &o.p->layouts[o.num_layouts++];
    memset(L, 0, sizeof(*L));
    for (int k = 0; k < c.rb; ++k) L->rb[k] = bits[k];
    L->first_gate = o.num_records;
    for (int gi : grp.second) layout_record(o, c, gi, local, kreg);
    L->num_gates = o.num_records - L->first_gate;
  }
  op->count = o.num_layouts - op->first;
}

}  // namespace

extern "C" int gbsv_plan(const gbsv_gate_desc_t* gates, int num_gates,
                         const void* matrices, int num_qubits,
                         int tile_qubits, int min_contiguous,
                         int register_bits, int fuse, gbsv_plan_t* plan) {
  if (!plan || (num_gates > 0 && (!gates || !matrices)))
    return GBSV_ERR_INVALID_ARG;
  const int n = num_qubits, m = tile_qubits;
  if (n < 1 || n > 62 || m < 1 || m > n || m > 14 || min_contiguous < 0 ||
      register_bits < 0 || register_bits > 5 ||
      (plan->dtype != GBSV_C64 && plan->dtype != GBSV_C128))
    return GBSV_ERR_INVALID_ARG;
  for (int i = 0; i < num_gates; ++i) {
    const gbsv_gate_desc_t& d = gates[i];
    if (d.nq < 1 || d.nq > 12 || d.q0 < 0 || d.q0 >= n ||
        (d.nq == 2 && (d.q1 < 0 || d.q1 >= n || d.q1 == d.q0)) ||
        d.kind < 0 || d.kind > 2 || d.mat < 0 || d.mat_bstride < 0)
      return GBSV_ERR_INVALID_ARG;
  }
  Ctx c{gates, static_cast<const cd*>(matrices), n, m,
        std::min(min_contiguous, m), register_bits};
  Out o;
  o.p = plan;
  const bool layouts =
      register_bits >= 1 && register_bits <= m && m <= register_bits + 9;
  const uint64_t low = c.c_min >= 64 ? ~0ull : ((uint64_t(1) << c.c_min) - 1);
  bool have = false;
  uint64_t tile = 0;
  std::vector<int> cur;
  auto close = [&]() {
    if (have) emit_stage(o, c, tile, cur, layouts);
    have = false;
    cur.clear();
  };
  for (int gi = 0; gi < num_gates && !o.overflow; ++gi) {
    int64_t need = fuse ? needs(c, gi) : -1;
    if (need >= 0 && popc(low | (uint64_t)need) > m) need = -1;
    if (need < 0) {
      close();
      if (o.num_ops >= plan->max_ops) {
        o.overflow = true;
        break;
      }
      gbsv_plan_op_t* op = &plan->ops[o.num_ops++];
      memset(op, 0, sizeof(*op));
      op->type = 0;
      op->first = gi;
      op->count = 1;
      continue;
    }
    if (!have) {
      have = true;
      tile = low;
    }
    if (popc(tile | (uint64_t)need) <= m) {
      tile |= (uint64_t)need;
      cur.push_back(gi);
    } else {
      close();
      have = true;
      tile = low | (uint64_t)need;
      cur.push_back(gi);
    }
  }
  close();
  if (o.overflow) return GBSV_ERR_SCRATCH;
  plan->num_ops = o.num_ops;
  plan->num_records = o.num_records;
  plan->num_layouts = o.num_layouts;
  plan->pool_len = o.pool_len;
  plan->used_layouts = layouts ? 1 : 0;
  return GBSV_OK;
}
