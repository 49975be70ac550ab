// Fork-join of independent big-number products on host helper threads.
//
// The reference orbit, the ball-arithmetic period search and the Newton
// nucleus refinement are serial in the iteration index, but each iteration
// performs several multiplications of the previous iterate's values that do not
// depend on one another (6 in a Newton step, 7 in a period-search step when
// its containment test lags one step, 2 in an orbit step). Up to six helpers. Running them at once on helper threads shortens each
// iteration; every product is the same GMP (or fixed-point) call on the same
// operands into a destination of the same precision, so results are bit for
// bit those of the serial loop. Helpers spin only while a session is open (a
// loop over iterations) and sleep otherwise.
#pragma once
#include <atomic>
#include <condition_variable>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

namespace mbx {

class ParMul {
  public:
    using Fn = void (*)(void* ctx, int k);
    static ParMul& instance();
    ~ParMul();
    // fn(ctx, k) for k in [0, n): k = 0 on the caller, the others on helpers.
    // Inside an open session and n <= width(); otherwise all run on the caller.
    void run(Fn fn, void* ctx, int n);
    // True when run(.., n) will execute its n calls concurrently (an open
    // session in the owning process with n <= width()): calls that wait on
    // one another may only be issued then.
    bool concurrent(int n) const;
    void open();
    void close();
    int width() const { return (int)helpers_.size() + 1; }

  private:
    ParMul();
    void helper(int h);
    struct alignas(64) Slot {
        std::atomic<unsigned> seq{0};
        std::atomic<unsigned> ack{0};
    };
    std::vector<std::thread> helpers_;
    std::unique_ptr<Slot[]> slots_;
    std::atomic<bool> open_{false}, quit_{false};
    std::mutex mu_;
    std::condition_variable cv_;
    int depth_ = 0;
    long pid_ = 0; // the process that owns the helpers
    Fn fn_ = nullptr;
    void* ctx_ = nullptr;
    int n_ = 0;
    unsigned round_ = 0;
};

// Keeps the helpers spinning for the lifetime of a loop when `enable`.
struct ParSession {
    bool on;
    explicit ParSession(bool enable) : on(enable) {
        if (on) ParMul::instance().open();
    }
    ~ParSession() {
        if (on) ParMul::instance().close();
    }
};

} // namespace mbx
