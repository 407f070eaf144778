// Stand-in for the HPX parallel algorithms NLMech calls (TEST INFRASTRUCTURE
// ONLY, oracle/refshim).  hpx::for_loop(policy, first, last, f) runs f(i)
// for i in [first, last) with an OpenMP loop; the task policy returns a
// future that is already ready.  Iterations are independent in every caller
// (each writes only its own row), as the reference's parallel loops require.
#pragma once

#include <cstdint>
#include <utility>

namespace boost {
using uint64_t = std::uint64_t;
}

namespace hpx {

struct ready_future {
  void get() const {}
  void wait() const {}
};

namespace execution {
struct task_policy_tag {};
inline constexpr task_policy_tag task{};
struct task_policy {};
struct parallel_policy {
  task_policy operator()(task_policy_tag) const { return {}; }
};
inline constexpr parallel_policy par{};
struct sequenced_policy {};
inline constexpr sequenced_policy seq{};
}  // namespace execution

namespace detail {
template <class I1, class I2, class F>
void run_loop(I1 first, I2 last, F &&f) {
  const long long a = (long long)first, b = (long long)last;
#pragma omp parallel for schedule(static)
  for (long long i = a; i < b; i++) f((boost::uint64_t)i);
}
}  // namespace detail

template <class I1, class I2, class F>
void for_loop(execution::parallel_policy, I1 first, I2 last, F &&f) {
  detail::run_loop(first, last, std::forward<F>(f));
}
template <class I1, class I2, class F>
void for_loop(execution::sequenced_policy, I1 first, I2 last, F &&f) {
  for (long long i = (long long)first; i < (long long)last; i++) f((boost::uint64_t)i);
}
template <class I1, class I2, class F>
ready_future for_loop(execution::task_policy, I1 first, I2 last, F &&f) {
  detail::run_loop(first, last, std::forward<F>(f));
  return {};
}

}  // namespace hpx
