// Oracle build support (test infrastructure only): a small stand-in for the
// part of the Taskflow library that the tinyvlm CPU backend uses, so that the
// reference's own backend sources (vlm/backends/cpu/src/vlm_backend_cpu.cpp,
// vlm_backend_cpud.cpp) compile unmodified without the network-fetched
// dependency.  It provides:
//   tf::Taskflow  placeholder(), emplace(callable), for_each_index(first, last, callable)
//   tf::Task      name(), precede(tasks...)
//   tf::Executor  Executor(threads), run(taskflow).wait()
// Execution follows Taskflow's documented rules for the graphs the backend
// builds: a task starts once all its strong predecessors are done; a
// condition task (a callable returning int) runs only successor number k and
// does not count as a strong predecessor, which is how the backend writes its
// loops (vlm_backend_cpu.cpp:121-139).  Tasks run one after another in a
// fixed order; a parallel-for task spreads its indices over OpenMP threads.
#pragma once

// the real library's headers bring these in, and the backend relies on it
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <deque>
#include <functional>
#include <memory>
#include <string>
#include <thread>
#include <type_traits>
#include <utility>
#include <vector>

namespace tf {

namespace detail {
struct Node {
    std::function<void()> work;     // plain or parallel-for task (may be empty)
    std::function<int()> cond;      // condition task
    bool is_cond = false;
    std::vector<Node*> succ;
    int strong_in = 0;              // predecessors that are not condition tasks
    int any_in = 0;                 // all predecessors
    std::string label;
    size_t idx = 0;                 // position in the owning graph
};
}  // namespace detail

class Task {
public:
    Task() = default;
    explicit Task(detail::Node* n) : n_(n) {}
    Task& name(const std::string& s) { n_->label = s; return *this; }
    template <class... Ts>
    Task& precede(Ts&&... ts) {
        (link(ts), ...);
        return *this;
    }
    detail::Node* node() const { return n_; }

private:
    void link(const Task& t) {
        n_->succ.push_back(t.n_);
        t.n_->any_in++;
        if (!n_->is_cond) t.n_->strong_in++;
    }
    detail::Node* n_ = nullptr;
};

class Taskflow {
public:
    Task placeholder() { return add(); }

    template <class C>
    Task emplace(C&& c) {
        Task t = add();
        using R = std::invoke_result_t<C&>;
        if constexpr (std::is_integral_v<R>) {
            t.node()->is_cond = true;
            t.node()->cond = std::function<int()>(std::forward<C>(c));
        } else {
            t.node()->work = std::function<void()>(std::forward<C>(c));
        }
        return t;
    }

    template <class B, class E, class C>
    Task for_each_index(B first, E last, C c) {
        const int64_t b = (int64_t)first, e = (int64_t)last;
        return emplace([b, e, c]() {
#pragma omp parallel for schedule(dynamic, 1)
            for (int64_t i = b; i < e; i++) c(i);
        });
    }

    template <class B, class E, class S, class C>
    Task for_each_index(B first, E last, S step, C c) {
        const int64_t b = (int64_t)first, e = (int64_t)last, s = (int64_t)step;
        return emplace([b, e, s, c]() {
            const int64_t n = s > 0 ? (e - b + s - 1) / s : 0;
#pragma omp parallel for schedule(dynamic, 1)
            for (int64_t k = 0; k < n; k++) c(b + k * s);
        });
    }

    // Runs the graph once to completion.
    void run_once() {
        std::vector<int> left(nodes_.size());
        std::deque<detail::Node*> ready;
        for (size_t i = 0; i < nodes_.size(); i++) {
            left[i] = nodes_[i]->strong_in;
            if (nodes_[i]->any_in == 0) ready.push_back(nodes_[i].get());
        }
        while (!ready.empty()) {
            detail::Node* n = ready.front();
            ready.pop_front();
            if (n->is_cond) {
                const int k = n->cond();
                if (k >= 0 && (size_t)k < n->succ.size()) ready.push_back(n->succ[(size_t)k]);
                continue;
            }
            if (n->work) n->work();
            for (detail::Node* s : n->succ)
                if (--left[s->idx] == 0) ready.push_back(s);
        }
    }

private:
    Task add() {
        nodes_.push_back(std::make_unique<detail::Node>());
        nodes_.back()->idx = nodes_.size() - 1;
        return Task(nodes_.back().get());
    }
    std::vector<std::unique_ptr<detail::Node>> nodes_;
};

class Future {
public:
    void wait() const {}
    void get() const {}
};

class Executor {
public:
    explicit Executor(size_t threads = std::thread::hardware_concurrency()) : threads_(threads) {}
    Future run(Taskflow& f) {
        f.run_once();
        return Future();
    }
    size_t num_workers() const { return threads_; }

private:
    size_t threads_;
};

}  // namespace tf
