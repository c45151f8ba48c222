// Sequential stand-in for the subset of HPX 1.10 that the LULESH task-based
// reference uses. It lets the unmodified reference sources compile and run
// without the HPX runtime, so that their numerical results can serve as the
// oracle for the GPU path.
//
// Test infrastructure only: nothing in the shipped library includes this.
//
// Semantics: every task runs eagerly on the calling thread at the point where
// it is created (hpx::async, future::then). The reference's task graph
// (lulesh.cc:1977-2240) only ever orders work through futures and
// when_all barriers, and every reduction it performs is a CSR-ordered sum or
// an exact min, so eager in-order execution gives the same bits as any
// parallel schedule of the same graph.
//
// Covered call sites (reference lulesh.cc):
//   async / then / shared_future   2029-2036, 2057-2067, 2104, 2127-2132, 2187-2198
//   when_all                       2040, 2073, 2112, 2138, 2204, 2229
//   unwrap_all / wait_all          2231 / 2239
//   for_each, transform, transform_reduce, reduce (execution::seq)
//                                  571-586, 1793, 1942, 1961, 2233
//   get_num_worker_threads         2346, 2405
#pragma once

#include <any>
#include <cstdint>
#include <functional>
#include <iomanip>
#include <iterator>
#include <limits>
#include <memory>
#include <sstream>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

namespace hpx {

namespace detail {
inline int& worker_threads() {
    static int n = 1;
    return n;
}
}  // namespace detail

inline int get_num_worker_threads() { return detail::worker_threads(); }

template <class T> class future;
template <class T> class shared_future;

namespace detail {
// Builds a ready future<R> from invoking f(args...), treating void results.
template <class F, class... A>
auto make_ready_from_call(F&& f, A&&... a);
}  // namespace detail

// A future that is always ready: the value was computed when it was created.
template <class T>
class future {
   public:
    using value_type = T;
    future() = default;
    explicit future(T v) : v_(std::make_shared<T>(std::move(v))) {}
    future(future&&) noexcept = default;
    future& operator=(future&&) noexcept = default;
    future(const future&) = delete;
    future& operator=(const future&) = delete;

    bool valid() const { return static_cast<bool>(v_); }
    T get() {
        std::shared_ptr<T> p = std::move(v_);
        return std::move(*p);
    }
    template <class F>
    auto then(F&& f) {
        return detail::make_ready_from_call(std::forward<F>(f), std::move(*this));
    }

   private:
    std::shared_ptr<T> v_;
    friend class shared_future<T>;
};

template <>
class future<void> {
   public:
    using value_type = void;
    future() = default;
    struct ready_tag {};
    explicit future(ready_tag) : ready_(true) {}
    future(future&&) noexcept = default;
    future& operator=(future&&) noexcept = default;
    future(const future&) = delete;
    future& operator=(const future&) = delete;

    bool valid() const { return ready_; }
    void get() { ready_ = false; }
    template <class F>
    auto then(F&& f) {
        return detail::make_ready_from_call(std::forward<F>(f), std::move(*this));
    }

   private:
    bool ready_ = false;
};

template <class T>
class shared_future {
   public:
    shared_future() = default;
    shared_future(future<T>&& f) : v_(std::move(f.v_)) {}
    const T& get() const { return *v_; }

   private:
    std::shared_ptr<T> v_;
};

template <>
class shared_future<void> {
   public:
    shared_future() = default;
    shared_future(future<void>&& f) : ready_(f.valid()) { f.get(); }
    void get() const {}

   private:
    bool ready_ = false;
};

namespace detail {
template <class F, class... A>
auto make_ready_from_call(F&& f, A&&... a) {
    using R = std::invoke_result_t<F, A...>;
    if constexpr (std::is_void_v<R>) {
        std::invoke(std::forward<F>(f), std::forward<A>(a)...);
        return future<void>(future<void>::ready_tag{});
    } else {
        return future<R>(std::invoke(std::forward<F>(f), std::forward<A>(a)...));
    }
}
}  // namespace detail

template <class F, class... A>
auto async(F&& f, A&&... a) {
    return detail::make_ready_from_call(std::forward<F>(f), std::forward<A>(a)...);
}

template <class T>
future<std::vector<future<T>>> when_all(std::vector<future<T>>& v) {
    return future<std::vector<future<T>>>(std::move(v));
}

template <class T>
future<std::vector<future<T>>> when_all(std::vector<future<T>>&& v) {
    return future<std::vector<future<T>>>(std::move(v));
}

template <class T>
void wait_all(std::vector<future<T>>&& v) {
    for (auto& f : v) f.get();
}

template <class T>
void wait_all(std::vector<future<T>>& v) {
    for (auto& f : v) f.get();
}

template <class T>
std::vector<T> unwrap_all(future<std::vector<future<T>>>& f) {
    std::vector<future<T>> inner = f.get();
    std::vector<T> out;
    out.reserve(inner.size());
    for (auto& x : inner) out.push_back(x.get());
    return out;
}

template <class T>
std::vector<T> unwrap_all(future<std::vector<future<T>>>&& f) {
    return unwrap_all(f);
}

namespace execution {
struct sequenced_policy {};
inline constexpr sequenced_policy seq{};
}  // namespace execution

template <class It, class F>
void for_each(execution::sequenced_policy, It first, It last, F&& f) {
    for (; first != last; ++first) f(*first);
}

// Binary transform, HPX argument order (first1, last1, first2, dest, op).
template <class It1, class It2, class Out, class F>
Out transform(execution::sequenced_policy, It1 first1, It1 last1, It2 first2, Out dest, F&& op) {
    for (; first1 != last1; ++first1, ++first2, ++dest) *dest = op(*first1, *first2);
    return dest;
}

// HPX argument order: (first, last, init, reduce_op, convert_op); left fold.
template <class It, class T, class Red, class Conv>
T transform_reduce(execution::sequenced_policy, It first, It last, T init, Red&& red, Conv&& conv) {
    for (; first != last; ++first) init = red(init, conv(*first));
    return init;
}

template <class It, class T, class Red>
T reduce(execution::sequenced_policy, It first, It last, T init, Red&& red) {
    for (; first != last; ++first) init = red(init, *first);
    return init;
}

}  // namespace hpx
