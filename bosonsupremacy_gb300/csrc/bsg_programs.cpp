// Host-side generation of partition programs for the repetition-aware
// hafnian (see bsg_internal.h for the recurrence).
#include <algorithm>
#include <cstring>
#include <string>
#include <unordered_map>

#include "bsg_internal.h"

namespace bsg {

// transition words pack (F slot << 9) | (b << 2): the byte offset of class b
// in a lane's int class array and, for 16-byte F entries, the byte offset of
// the source slot's [32 lanes] row.  Every transition of a state shares its
// first class a, which the state's pack word carries.
static_assert(BSG_MAX_CLASSES <= 32, "class byte offsets take bits 2..6 of a transition word");
static_assert(BSG_MAX_CLASSES < 256 && kKeyMaxMult + 1 < 256, "transition counts and r_a take 8 bits of a pack word");
static_assert(2 * BSG_MAX_STATES < (1 << 23), "F ring slots take 23 bits of a transition word");

int key_order(uint64_t key) {
  int n = 0;
  for (int v = 1; v <= kKeyMaxMult; ++v) n += v * int((key >> (kKeyBits * (v - 1))) & 63);
  return n;
}

int key_classes(uint64_t key) {
  int k = 0;
  for (int v = 1; v <= kKeyMaxMult; ++v) k += int((key >> (kKeyBits * (v - 1))) & 63);
  return k;
}

// The program of one key, built apart from the program set (thread-safe:
// the planner builds the new keys of a build in parallel and appends them in
// a fixed order).  On failure b.err holds the status and b.msg the message.
int build_program(uint64_t key, ProgramBuild& b) {
  // site programs: jroot = jmax >= 0 (the site class last, roots at jmax, jmax - 2, ...)
  const int jroot = int(key >> kKeyRootShift) - 1;
  const uint64_t xkey = key & ((uint64_t(1) << kKeyRootShift) - 1);
  std::vector<int>& mult = b.mult;
  mult.clear();
  for (int v = 1; v <= kKeyMaxMult; ++v) {
    int c = int((xkey >> (kKeyBits * (v - 1))) & 63);
    for (int i = 0; i < c; ++i) mult.push_back(v);
  }
  if (jroot >= 0) mult.push_back(jroot);
  const int k = int(mult.size());
  b.k = k;
  if (k > BSG_MAX_CLASSES) {
    b.err = BSG_ERR_LIMIT;
    b.msg = "hafnian with " + std::to_string(k) + " distinct indices exceeds BSG_MAX_CLASSES=" +
            std::to_string(BSG_MAX_CLASSES);
    return b.err;
  }
  // Enumerate the states reachable from the root(s).
  std::unordered_map<std::string, int> seen;
  std::vector<std::string> states;
  std::vector<std::string> stack;
  std::string full(k, '\0');
  for (int c = 0; c < k; ++c) full[c] = char(mult[c]);
  std::unordered_map<std::string, int> root_j;  // root state -> its site multiplicity
  if (jroot >= 0) {
    for (int j = jroot; j >= 0; j -= 2) {
      std::string r = full;
      r[k - 1] = char(j);
      root_j.emplace(r, j);
      stack.push_back(r);
    }
  } else {
    stack.push_back(full);
  }
  while (!stack.empty()) {
    std::string st = std::move(stack.back());
    stack.pop_back();
    if (seen.count(st)) continue;
    seen.emplace(st, int(states.size()));
    states.push_back(st);
    if (int(states.size()) > BSG_MAX_STATES) {
      b.err = BSG_ERR_LIMIT;
      b.msg = "partition with " + std::to_string(k) + " classes (n=" +
              std::to_string(key_order(xkey) + std::max(jroot, 0)) + ") needs more than BSG_MAX_STATES=" +
              std::to_string(BSG_MAX_STATES) + " DP states";
      return b.err;
    }
    int a = 0;
    while (a < k && st[a] == 0) ++a;
    if (a == k) continue;
    for (int c = a; c < k; ++c) {
      if (st[c] == 0 || (c == a && st[a] < 2)) continue;
      std::string t = st;
      t[a]--;
      t[c]--;
      if (!seen.count(t)) stack.push_back(t);
    }
  }
  // Topological order: ascending total (every transition removes two units).
  auto total = [](const std::string& x) {
    int t = 0;
    for (char c : x) t += c;
    return t;
  };
  std::vector<int> order(states.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = int(i);
  std::stable_sort(order.begin(), order.end(),
                   [&](int x, int y) { return total(states[x]) < total(states[y]); });
  std::vector<int> local(states.size());
  for (size_t i = 0; i < order.size(); ++i) local[order[i]] = int(i);
  // F ring slots: a state of total T reads only states of total T - 2, so
  // two levels of F are live at a time; slot = (level % 2) * W + position in
  // level, W = the widest level.
  std::vector<int> slot(states.size());
  int width = 1;
  {
    std::vector<int> level_count;
    std::vector<int> pos(states.size());
    const int t0 = total(states[order[0]]);
    for (size_t i = 0; i < order.size(); ++i) {
      const int lv = (total(states[order[i]]) - t0) / 2;
      if (lv >= (int)level_count.size()) level_count.resize(lv + 1, 0);
      pos[i] = level_count[lv]++;
    }
    for (int c : level_count) width = std::max(width, c);
    for (size_t i = 0; i < order.size(); ++i) {
      const int lv = (total(states[order[i]]) - t0) / 2;
      slot[i] = (lv & 1) * width + pos[i];
    }
  }
  b.nstates = int(states.size());
  b.fslots = states.size() > 1 ? 2 * width : 1;
  b.trans.clear();
  b.st_trans_off.clear();
  b.st_trans_cnt.clear();
  b.st_ra.clear();
  b.st_pack.clear();
  for (size_t i = 0; i < order.size(); ++i) {
    const std::string& st = states[order[i]];
    b.st_trans_off.push_back(int(b.trans.size()));  // relative to the program's first transition
    int a = 0;
    while (a < k && st[a] == 0) ++a;
    int cnt = 0;
    if (a < k) {
      for (int c = a; c < k; ++c) {
        if (st[c] == 0 || (c == a && st[a] < 2)) continue;
        std::string t = st;
        t[a]--;
        t[c]--;
        const uint32_t src = uint32_t(slot[local[seen.at(t)]]);
        b.trans.push_back((src << 9) | (uint32_t(c) << 2));
        ++cnt;
      }
    }
    b.st_trans_cnt.push_back(cnt);
    b.st_ra.push_back(a < k ? int(st[a]) : 0);
    auto rj = root_j.find(st);
    const uint32_t tag = rj == root_j.end() ? 0u : uint32_t(rj->second + 1);
    b.st_pack.push_back(make_uint4(uint32_t(b.st_trans_off.back()),
                                   uint32_t(cnt) | (uint32_t(a < k ? st[a] : 0) << 8) | (tag << 16),
                                   uint32_t(slot[i]), uint32_t(a < k ? a : 0)));
  }
  b.err = BSG_OK;
  return BSG_OK;
}

// Appends a built program to the set (serial); returns its index.
int append_program(ProgramSet& ps, uint64_t key, const ProgramBuild& b) {
  const int prog = int(ps.keys.size());
  const int base = int(ps.st_trans_off.size());
  const uint32_t toff = uint32_t(ps.trans.size());
  ps.keys.push_back(key);
  ps.k.push_back(b.k);
  ps.nstates.push_back(b.nstates);
  ps.state_off.push_back(base);
  ps.fslots.push_back(b.fslots);
  for (int c = 0; c < BSG_MAX_CLASSES; ++c) ps.mult.push_back(c < b.k ? b.mult[c] : 0);
  for (int i = 0; i < b.nstates; ++i) {
    ps.st_trans_off.push_back(int(toff) + b.st_trans_off[i]);
    ps.st_trans_cnt.push_back(b.st_trans_cnt[i]);
    ps.st_ra.push_back(b.st_ra[i]);
    uint4 pk = b.st_pack[i];
    pk.x += toff;
    ps.st_pack.push_back(pk);
  }
  ps.trans.insert(ps.trans.end(), b.trans.begin(), b.trans.end());
  ps.index.emplace(key, prog);
  ps.max_states = std::max(ps.max_states, b.nstates);
  ps.max_k = std::max(ps.max_k, b.k);
  ps.dev_valid = false;
  return prog;
}

int program_for_key(ProgramSet& ps, uint64_t key, int32_t* prog_out) {
  auto it = ps.index.find(key);
  if (it != ps.index.end()) {
    *prog_out = it->second;
    return BSG_OK;
  }
  ProgramBuild b;
  if (build_program(key, b) != BSG_OK) {
    set_error("%s", b.msg.c_str());
    return b.err;
  }
  *prog_out = append_program(ps, key, b);
  return BSG_OK;
}

// Appends v[done:] to the device copy; a copy that must grow is reallocated
// (cudaFree waits for the device, so no launch still reads the old one) and
// refilled.  Entries already on the device are never rewritten, so launches
// in flight on other streams keep reading valid programs.
template <class T>
static int upload(T*& dptr, size_t& cap, size_t done, const std::vector<T>& v, cudaStream_t stream) {
  size_t need = std::max<size_t>(v.size(), 1);
  if (need > cap) {
    if (dptr) cudaFree(dptr);
    dptr = nullptr;
    size_t c = std::max(need, cap * 2);
    BSG_CUDA(cudaMalloc(&dptr, c * sizeof(T)));
    cap = c;
    done = 0;
  }
  if (v.size() > done)
    BSG_CUDA(cudaMemcpyAsync(dptr + done, v.data() + done, (v.size() - done) * sizeof(T), cudaMemcpyHostToDevice,
                             stream));
  return BSG_OK;
}

int programs_upload(ProgramSet& ps, cudaStream_t stream) {
  if (ps.dev_valid) return BSG_OK;
  size_t pc = ps.dev_prog_cap, pc2 = ps.dev_prog_cap, pc3 = ps.dev_prog_cap;
  BSG_TRY(upload(ps.d_k, pc, ps.dev_prog_n, ps.k, stream));
  BSG_TRY(upload(ps.d_nstates, pc2, ps.dev_prog_n, ps.nstates, stream));
  BSG_TRY(upload(ps.d_state_off, pc3, ps.dev_prog_n, ps.state_off, stream));
  ps.dev_prog_cap = pc;
  ps.dev_prog_n = ps.k.size();
  size_t sc = ps.dev_states_cap;
  BSG_TRY(upload(ps.d_st_pack, sc, ps.dev_states_n, ps.st_pack, stream));
  ps.dev_states_cap = sc;
  ps.dev_states_n = ps.st_trans_off.size();
  BSG_TRY(upload(ps.d_trans, ps.dev_trans_cap, ps.dev_trans_n, ps.trans, stream));
  ps.dev_trans_n = ps.trans.size();
  // Copies from these pageable vectors are staged before cudaMemcpyAsync
  // returns, so the host may append programs right away.
  ps.dev_valid = true;
  return BSG_OK;
}

void programs_free(ProgramSet& ps) {
  cudaFree(ps.d_k);
  cudaFree(ps.d_nstates);
  cudaFree(ps.d_state_off);
  cudaFree(ps.d_st_pack);
  cudaFree(ps.d_trans);
  ps = ProgramSet();
}

}  // namespace bsg
