/*
 * clemu_rt.cpp — TEST INFRASTRUCTURE.  Execution model of the OpenCL-C
 * emulation: kernels registered by name, NDRange launches with work-groups in
 * row-major order (rows of groups spread over OpenMP threads), and work-items
 * of a group run as fibers in raster order so that barrier() suspends each
 * item until all items of the group reach it.  Fibers start on their own
 * stacks through makecontext and switch with swapcontext.
 */
#include <ucontext.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <memory>
#include <mutex>

#include "clemu.h"

namespace clemu {

thread_local WorkItem* t_item = nullptr;
std::function<void(const std::string&, const std::vector<Arg>&)> on_launch;

namespace {

struct Entry { bool barrier; ItemFn fn; };
std::map<std::string, Entry>& registry() { static std::map<std::string, Entry> r; return r; }

const size_t STACK = 256 * 1024;

struct Fiber {
    ucontext_t uc;
    char* stack = nullptr;
    int state = 0;            /* 0 fresh, 1 at a barrier, 2 done, 3 running */
    WorkItem wi;
};

struct Sched {
    std::vector<Fiber> fibers;
    std::vector<char> stacks;
    ucontext_t uc;
    Fiber* cur = nullptr;
    const ItemFn* fn = nullptr;
    const std::vector<Arg>* args = nullptr;
};

thread_local Sched* t_sched = nullptr;
thread_local std::vector<std::vector<char>> t_arena;

/* Every switch between the scheduler and a work-item goes through
 * swapcontext/setcontext, which also switch the shadow stack of processes
 * that run with one (a longjmp onto another stack does not). */
void trampoline() {
    Sched* s = t_sched;
    (*s->fn)(*s->args);
    s->cur->state = 2;
    setcontext(&s->uc);
}

void resume(Sched* s, Fiber* f) {
    s->cur = f;
    t_item = &f->wi;
    if (f->state == 0) {
        getcontext(&f->uc);
        f->uc.uc_stack.ss_sp = f->stack;
        f->uc.uc_stack.ss_size = STACK;
        f->uc.uc_link = nullptr;
        makecontext(&f->uc, trampoline, 0);
    }
    f->state = 3;
    swapcontext(&s->uc, &f->uc);
}

}  // namespace

void barrier(int) {
    Sched* s = t_sched;
    if (!s) { fprintf(stderr, "clemu: barrier() in a kernel registered without barriers\n"); abort(); }
    Fiber* f = s->cur;
    f->state = 1;
    swapcontext(&f->uc, &s->uc);
}

/* Local memory of argument `index`, 64-byte aligned: the kernels' local
 * float8 buffers are 32-byte aligned types, and vector code may use aligned
 * loads on them (std::vector storage alone guarantees only 16 bytes). */
void* local_arena(int index, size_t bytes) {
    if ((int)t_arena.size() <= index) t_arena.resize(index + 1);
    std::vector<char>& a = t_arena[index];
    if (a.size() < bytes + 64) a.assign(bytes + 64, 0);
    return (void*)(((uintptr_t)a.data() + 63) & ~(uintptr_t)63);
}

void reg(const std::string& name, bool uses_barrier, ItemFn fn) { registry()[name] = Entry{uses_barrier, fn}; }
bool has_kernel(const std::string& name) { return registry().count(name) != 0; }

void launch(const std::string& name, const std::vector<Arg>& args, size_t gx, size_t gy, size_t lx, size_t ly) {
    launch3(name, args, gx, gy, 1, lx, ly);
}

void launch3(const std::string& name, const std::vector<Arg>& args, size_t gx, size_t gy, size_t gz, size_t lx,
             size_t ly) {
    auto it = registry().find(name);
    if (it == registry().end()) { fprintf(stderr, "clemu: unknown kernel %s\n", name.c_str()); abort(); }
    const Entry& e = it->second;
    if (gx % lx || gy % ly) { fprintf(stderr, "clemu: global size not a multiple of local size\n"); abort(); }
    const long ngx = (long)(gx / lx), ngy = (long)(gy / ly), ngz = (long)gz;
    const int n = (int)(lx * ly);
#pragma omp parallel for schedule(dynamic, 1)
    for (long gyz = 0; gyz < ngy * ngz; ++gyz) {
        const long gyi = gyz % ngy, gzi = gyz / ngy;   /* z-planes of groups one after another */
        static thread_local std::unique_ptr<Sched> sched;
        if (!sched || (int)sched->fibers.size() < n) {
            sched.reset(new Sched());
            sched->fibers.resize(n);
            sched->stacks.assign((size_t)n * STACK, 0);
            for (int i = 0; i < n; ++i) sched->fibers[i].stack = sched->stacks.data() + (size_t)i * STACK;
        }
        Sched* s = sched.get();
        s->fn = &e.fn;
        s->args = &args;
        for (long gxi = 0; gxi < ngx; ++gxi) {
            for (int i = 0; i < n; ++i) {
                WorkItem& w = s->fibers[i].wi;
                w.lid[0] = i % lx; w.lid[1] = i / lx; w.lid[2] = 0;
                w.grp[0] = gxi; w.grp[1] = gyi; w.grp[2] = gzi;
                w.lsz[0] = lx; w.lsz[1] = ly; w.lsz[2] = 1;
                w.gid[0] = gxi * lx + w.lid[0]; w.gid[1] = gyi * ly + w.lid[1]; w.gid[2] = gzi;
                s->fibers[i].state = 0;
            }
            if (!e.barrier) {
                t_sched = nullptr;
                for (int i = 0; i < n; ++i) { t_item = &s->fibers[i].wi; e.fn(args); }
                continue;
            }
            t_sched = s;
            for (;;) {
                bool left = false;
                for (int i = 0; i < n; ++i)
                    if (s->fibers[i].state != 2) { resume(s, &s->fibers[i]); left = true; }
                if (!left) break;
            }
            t_sched = nullptr;
        }
    }
    if (on_launch) on_launch(name, args);
}

}  // namespace clemu
