/*
 * NDRange execution on the CPU for the reference's OpenCL kernels compiled
 * through oracle/ref_stubs/opencl_c.hpp.  TEST INFRASTRUCTURE ONLY.
 *
 * An NDRange runs one work-group after another.  Within a group, kernels with
 * barriers run their work-items as coroutines (ucontext) in turn: each runs
 * until its next barrier() or its end, so a barrier completes when every
 * work-item of the group has reached it (the kernels' barriers are uniform
 * over the group, as OpenCL requires).  Kernels without barriers run their
 * work-items one after another.  Work-group `local` arrays are function
 * statics, shared by the group and rewritten by each group before use.
 */
#include <ucontext.h>

#include <stdexcept>
#include <vector>

#include "opencl_c.hpp"

namespace clshim {
Ids* g_cur = nullptr;

namespace {
struct Coro {
    ucontext_t ctx;
    Ids ids;
    bool done;
};
ucontext_t g_sched;
Coro* g_running = nullptr;
bool g_in_coro = false;
void (*g_body)(void*) = nullptr;
void* g_body_arg = nullptr;

void trampoline() {
    g_body(g_body_arg);
    g_running->done = true;
    swapcontext(&g_running->ctx, &g_sched);
}

Ids ids_1d(size_t g, size_t l, size_t groups, size_t local_size, size_t global_size) {
    return Ids{{g * local_size + l, 0}, {l, 0}, {g, 0}, {groups, 1}, {local_size, 1}, {global_size, 1}};
}
}  // namespace

void barrier_yield() {
    if (!g_in_coro) throw std::logic_error("barrier() in a kernel launched without coroutines");
    swapcontext(&g_running->ctx, &g_sched);
}

void launch(size_t global_size, size_t local_size, bool barriers, void (*body)(void*), void* arg) {
    if (local_size == 0 || global_size % local_size) throw std::invalid_argument("NDRange not a multiple of the group");
    const size_t groups = global_size / local_size;
    if (!barriers) {
        Ids ids{};
        g_cur = &ids;
        for (size_t g = 0; g < groups; ++g)
            for (size_t l = 0; l < local_size; ++l) {
                ids = ids_1d(g, l, groups, local_size, global_size);
                body(arg);
            }
        g_cur = nullptr;
        return;
    }
    constexpr size_t kStack = 64 * 1024;
    std::vector<Coro> items(local_size);
    std::vector<char> stacks(kStack * local_size);
    g_body = body;
    g_body_arg = arg;
    g_in_coro = true;
    for (size_t g = 0; g < groups; ++g) {
        for (size_t l = 0; l < local_size; ++l) {
            Coro& c = items[l];
            c.ids = ids_1d(g, l, groups, local_size, global_size);
            c.done = false;
            getcontext(&c.ctx);
            c.ctx.uc_stack.ss_sp = stacks.data() + l * kStack;
            c.ctx.uc_stack.ss_size = kStack;
            c.ctx.uc_link = nullptr;
            makecontext(&c.ctx, trampoline, 0);
        }
        size_t left = local_size;
        while (left) {  // one round: every unfinished work-item runs to its next barrier or its end
            for (size_t l = 0; l < local_size; ++l) {
                Coro& c = items[l];
                if (c.done) continue;
                g_running = &c;
                g_cur = &c.ids;
                swapcontext(&g_sched, &c.ctx);
                if (c.done) --left;
            }
        }
    }
    g_in_coro = false;
    g_running = nullptr;
    g_cur = nullptr;
}

void launch2d(size_t gx, size_t gy, void (*body)(void*), void* arg) {
    Ids ids{};
    g_cur = &ids;
    for (size_t y = 0; y < gy; ++y)
        for (size_t x = 0; x < gx; ++x) {
            ids = Ids{{x, y}, {0, 0}, {x, y}, {gx, gy}, {1, 1}, {gx, gy}};
            body(arg);
        }
    g_cur = nullptr;
}
}  // namespace clshim
