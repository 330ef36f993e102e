// Minimal HClib-Actor "Selector" surface for compiling DAKC's counting sources
// (dakc/src/kcounter/kcounter.hpp:47-70, kcounter.cpp:263-300) on one host.
// Test infrastructure for the oracle only.
//
// Semantics kept: send(mb, pkt, pe) delivers pkt to PE pe's mailbox handler
// mb[mb].process(pkt, sender) exactly once, and hclib::finish returns only
// after every PE called done() and every message was processed.  Delivery is
// deferred to the end of finish (all sends, barrier, then each PE processes
// its inbox in sender order).  DAKC's result does not depend on delivery
// order: the receive side only appends, and phase 2 sorts.
#ifndef DK_SHIM_SELECTOR_H
#define DK_SHIM_SELECTOR_H
#include <functional>
#include <vector>
#include <cstdint>
#include <cstddef>
#include <cstring>

namespace dkshim {
// Blob exchange between forked PEs (implemented in dk_shim.cpp): every PE
// passes one byte buffer per destination; returns the buffers addressed to
// this PE, indexed by sender.
std::vector<std::vector<char>> exchange(const std::vector<std::vector<char>>& outgoing);
int my_pe();
int n_pes();
void barrier();
struct SelectorBase {
  virtual void deliver_all() = 0;
  virtual ~SelectorBase() {}
};
extern SelectorBase* g_active;
extern uint64_t g_items_received;  // items delivered to this PE (all mailboxes)
}  // namespace dkshim

namespace hclib {

template <int N, typename T>
class Selector : public dkshim::SelectorBase {
 public:
  struct Mailbox {
    std::function<void(T, int)> process;
  };
  Mailbox mb[N];

  Selector() : out_(N) {}
  void start() {
    for (int m = 0; m < N; ++m) out_[m].assign(dkshim::n_pes(), std::vector<T>());
    dkshim::g_active = this;
  }
  void send(int m, T pkt, int pe) { out_[m][pe].push_back(pkt); }
  void done(int /*m*/) {}

  void deliver_all() override {
    for (int m = 0; m < N; ++m) {
      const int P = dkshim::n_pes();
      std::vector<std::vector<char>> blobs(P);
      for (int pe = 0; pe < P; ++pe) {
        const auto& v = out_[m][pe];
        blobs[pe].resize(v.size() * sizeof(T));
        if (!v.empty()) std::memcpy(blobs[pe].data(), v.data(), blobs[pe].size());
        out_[m][pe].clear();
        out_[m][pe].shrink_to_fit();
      }
      std::vector<std::vector<char>> in = dkshim::exchange(blobs);
      for (int src = 0; src < P; ++src) {
        const size_t cnt = in[src].size() / sizeof(T);
        for (size_t i = 0; i < cnt; ++i) {
          T pkt;
          std::memcpy(&pkt, in[src].data() + i * sizeof(T), sizeof(T));
          dkshim::g_items_received += 1;
          mb[m].process(pkt, src);
        }
      }
    }
  }

 private:
  std::vector<std::vector<std::vector<T>>> out_;  // [mailbox][dest] -> packets
};

template <typename F>
void finish(F&& f) {
  dkshim::g_active = nullptr;
  f();
  if (dkshim::g_active) dkshim::g_active->deliver_all();
  dkshim::g_active = nullptr;
  dkshim::barrier();
}

}  // namespace hclib
#endif
