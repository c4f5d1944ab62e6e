// CPU-thread model of the offer_kill / groups_to_kill protocol.  Host
// threads play the persistent groups and the scheduler over the SAME
// protocol code the kernels run (wgm_protocol.h), with host atomics.  Built
// and driven by tests/test_protocol_model.py; test code only.
//
// A planted mistake lives here, never in the product: kRacy replaces the
// compare-and-swap decrement with the reference's load-then-store form
// (scheduler_1.cl:67-71), so the tests can show that they catch the stale
// store.
#include <atomic>
#include <chrono>
#include <cstdint>
#include <random>
#include <thread>
#include <vector>

#include "../../include/wgm_protocol.h"

namespace {

thread_local void (*g_hook)(void *) = nullptr;
thread_local void *g_hook_arg = nullptr;

struct HostOps {
  static int ld_acquire(int *p) { return std::atomic_ref<int>(*p).load(std::memory_order_acquire); }
  static int cas(int *p, int cmp, int v) {
    std::atomic_ref<int>(*p).compare_exchange_strong(cmp, v, std::memory_order_acq_rel,
                                                     std::memory_order_acquire);
    return cmp;  // the old value either way
  }
  static int add(int *p, int v) {
    return std::atomic_ref<int>(*p).fetch_add(v, std::memory_order_acq_rel);
  }
  static void between() {
    if (g_hook) g_hook(g_hook_arg);
    else std::this_thread::yield();
  }
};

// The planted mistake: read, then store the read value minus one.
bool racy_offer_kill(int *num_groups, int *to_kill, int kid) {
  if (kid != HostOps::ld_acquire(num_groups) - 1) return false;
  const int tk = HostOps::ld_acquire(to_kill);
  if (tk <= 0) return false;
  HostOps::between();
  std::atomic_ref<int>(*to_kill).store(tk - 1, std::memory_order_relaxed);
  HostOps::add(num_groups, -1);
  return true;
}

bool offer_kill(int racy, int *num_groups, int *to_kill, int kid) {
  return racy ? racy_offer_kill(num_groups, to_kill, kid)
              : wgm_proto_offer_kill<HostOps>(num_groups, to_kill, kid);
}

void clear_word(void *p) { std::atomic_ref<int>(*static_cast<int *>(p)).store(0); }

// Widens the window between a group's read and its decrement, so the
// scheduler's withdrawals land inside it often.
void short_pause(void *) { std::this_thread::sleep_for(std::chrono::microseconds(3)); }

}  // namespace

// The scheduler clears groups_to_kill (a waiting request got its groups
// elsewhere) between the highest group's read and its decrement.  out[0]:
// killed, out[1]: groups_to_kill afterwards, out[2]: group count afterwards.
extern "C" int model_kill_clear_interleaving(int racy, int *out) {
  int num_groups = 5, to_kill = 3;
  g_hook = clear_word;
  g_hook_arg = &to_kill;
  const bool killed = offer_kill(racy, &num_groups, &to_kill, 4);
  g_hook = nullptr;
  out[0] = killed;
  out[1] = to_kill;
  out[2] = num_groups;
  return 0;
}

// Stress: `groups` threads offer kills in a loop (thread i is persistent id
// i and leaves when killed); a scheduler thread asks for 1..3 groups at a
// time and, half of the time, withdraws the request before it is met.  After
// the last withdrawal the groups keep offering for a while.
//   out[0]  kills in all
//   out[1]  kills the scheduler's requests account for (each kill must
//           consume one unit of an outstanding request)
//   out[2]  kills after the final clear (must be 0)
//   out[3]  final group count
//   out[4]  ids that left out of order (must be 0: only the highest leaves)
//   out[5]  rounds that found a withdrawn request back in the word (must be 0)
extern "C" int model_kill_stress(int racy, int groups, int rounds, uint64_t seed, int64_t *out) {
  int num_groups = groups, to_kill = 0;
  std::atomic<int> phase{0};  // 0 running, 1 final clear done, 2 stop
  std::atomic<int64_t> kills{0}, late{0}, disorder{0};
  std::atomic<int> last_left{groups};
  std::vector<std::thread> th;
  for (int id = 1; id < groups; id++) {  // id 0 is the master, never killed
    th.emplace_back([&, id] {
      g_hook = short_pause;
      while (phase.load() < 2) {
        if (offer_kill(racy, &num_groups, &to_kill, id)) {
          kills++;
          if (phase.load() >= 1) late++;
          int prev = last_left.exchange(id);
          if (id != prev - 1) disorder++;
          return;
        }
        std::this_thread::yield();
      }
    });
  }
  std::mt19937_64 rng(seed);
  int64_t granted = 0;
  int64_t revived = 0;
  for (int r = 0; r < rounds; r++) {
    // the word was cleared at the end of the last round: anything else now
    // is a stale decrement that brought a withdrawn request back
    if (HostOps::ld_acquire(&to_kill) != 0) revived++;
    const int before = HostOps::ld_acquire(&num_groups);
    const int want = 1 + (int)(rng() % 3);
    std::atomic_ref<int>(to_kill).store(want, std::memory_order_release);
    if (rng() & 1) std::this_thread::sleep_for(std::chrono::microseconds(rng() % 50));
    else std::this_thread::yield();
    std::atomic_ref<int>(to_kill).store(0, std::memory_order_release);  // withdraw
    granted += before - HostOps::ld_acquire(&num_groups);
    if (HostOps::ld_acquire(&num_groups) <= 2) break;
  }
  // let in-flight offers finish, then count what the word still says
  std::this_thread::sleep_for(std::chrono::milliseconds(2));
  const int before_final = HostOps::ld_acquire(&num_groups);
  phase.store(1);
  std::this_thread::sleep_for(std::chrono::milliseconds(20));
  phase.store(2);
  for (auto &t : th) t.join();
  (void)before_final;
  out[0] = kills.load();
  out[1] = granted;
  out[2] = late.load();
  out[3] = num_groups;
  out[4] = disorder.load();
  out[5] = revived + (HostOps::ld_acquire(&to_kill) != 0);
  return 0;
}
