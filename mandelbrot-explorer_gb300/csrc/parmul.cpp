// ParMul (parmul.h): helpers wait on a condition variable while no session is
// open and spin on their slot's round counter while one is.
#include "parmul.h"

#include <unistd.h>

#include <algorithm>

namespace mbx {

// One pool per calling thread: engines building references on different
// threads (a batch) each get their own helpers.
ParMul& ParMul::instance() {
    thread_local ParMul p;
    return p;
}

ParMul::ParMul() {
    pid_ = (long)getpid();
    const unsigned hw = std::thread::hardware_concurrency();
    const int n = (int)std::min(6u, hw > 1 ? hw - 1 : 0u);
    slots_.reset(new Slot[n > 0 ? n : 1]);
    for (int h = 0; h < n; ++h) helpers_.emplace_back(&ParMul::helper, this, h);
}

ParMul::~ParMul() {
    {
        std::lock_guard<std::mutex> l(mu_);
        quit_.store(true);
        open_.store(false);
    }
    cv_.notify_all();
    for (auto& t : helpers_) t.join();
}

void ParMul::open() {
    if ((long)getpid() != pid_) return; // a forked child has no helper threads
    std::lock_guard<std::mutex> l(mu_);
    if (depth_++ == 0) open_.store(true, std::memory_order_release);
    cv_.notify_all();
}

void ParMul::close() {
    if ((long)getpid() != pid_) return;
    std::lock_guard<std::mutex> l(mu_);
    if (--depth_ == 0) open_.store(false, std::memory_order_release);
}

void ParMul::helper(int h) {
    Slot& s = slots_[h];
    unsigned seen = 0;
    for (;;) {
        {
            std::unique_lock<std::mutex> l(mu_);
            cv_.wait(l, [&] { return open_.load() || quit_.load(); });
            if (quit_.load()) return;
        }
        while (open_.load(std::memory_order_acquire)) {
            const unsigned r = s.seq.load(std::memory_order_acquire);
            if (r == seen) continue;
            seen = r;
            fn_(ctx_, h + 1);
            s.ack.store(r, std::memory_order_release);
        }
    }
}

bool ParMul::concurrent(int n) const { return n > 1 && n <= width() && open_.load(std::memory_order_acquire) && (long)getpid() == pid_; }

void ParMul::run(Fn fn, void* ctx, int n) {
    if (!concurrent(n)) {
        for (int k = 0; k < n; ++k) fn(ctx, k);
        return;
    }
    fn_ = fn;
    ctx_ = ctx;
    n_ = n;
    const unsigned r = ++round_;
    for (int h = 0; h < n - 1; ++h) slots_[h].seq.store(r, std::memory_order_release);
    fn(ctx, 0);
    for (int h = 0; h < n - 1; ++h)
        while (slots_[h].ack.load(std::memory_order_acquire) != r) {
        }
}

} // namespace mbx
