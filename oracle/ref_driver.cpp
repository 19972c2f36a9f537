// ref_driver.cpp -- runs the reference's own mpimg_* entry points
// (src/millipyde_image.cpp, compiled against oracle/ref_shim) on host
// buffers, and the coroutine scheduler behind the shim's kernel launches.
// Test infrastructure: produces golden vectors, never product code.
#include <ucontext.h>
#include <stdio.h>
#include <vector>

#include "hip/hip_runtime.h"
#include "millipyde.h"
#include "millipyde_image.h"

dim3 mpemu_tid, mpemu_bid, mpemu_bdim, mpemu_gdim;

namespace {
struct Fiber {
    ucontext_t ctx;
    std::vector<char> stack;
    bool done = false;
    bool at_barrier = false;
    unsigned tx, ty, tz;
};
ucontext_t g_sched;
Fiber *g_cur = nullptr;
std::function<void()> *g_body = nullptr;

void fiber_entry()
{
    (*g_body)();
    g_cur->done = true;
    swapcontext(&g_cur->ctx, &g_sched);
}
}  // namespace

void mpemu_syncthreads()
{
    g_cur->at_barrier = true;
    swapcontext(&g_cur->ctx, &g_sched);
}

void mpemu_launch(dim3 grid, dim3 block, std::function<void()> body)
{
    const unsigned nthreads = block.x * block.y * block.z;
    std::vector<Fiber> fibers(nthreads);
    g_body = &body;
    mpemu_gdim = grid;
    mpemu_bdim = block;
    for (unsigned bz = 0; bz < grid.z; ++bz)
        for (unsigned by = 0; by < grid.y; ++by)
            for (unsigned bx = 0; bx < grid.x; ++bx) {
                mpemu_bid = dim3(bx, by, bz);
                for (unsigned t = 0; t < nthreads; ++t) {
                    Fiber &f = fibers[t];
                    f.done = false;
                    f.at_barrier = false;
                    f.tx = t % block.x;
                    f.ty = (t / block.x) % block.y;
                    f.tz = t / (block.x * block.y);
                    f.stack.resize(64 * 1024);
                    getcontext(&f.ctx);
                    f.ctx.uc_stack.ss_sp = f.stack.data();
                    f.ctx.uc_stack.ss_size = f.stack.size();
                    f.ctx.uc_link = nullptr;
                    makecontext(&f.ctx, fiber_entry, 0);
                }
                // run every fiber to its next barrier (or its end), then release the barrier
                for (;;) {
                    bool any_waiting = false;
                    for (unsigned t = 0; t < nthreads; ++t) {
                        Fiber &f = fibers[t];
                        if (f.done) continue;
                        f.at_barrier = false;
                        g_cur = &f;
                        mpemu_tid = dim3(f.tx, f.ty, f.tz);
                        swapcontext(&g_sched, &f.ctx);
                        if (!f.done) any_waiting = true;
                    }
                    if (!any_waiting) break;
                }
            }
}

extern "C" {

// Runs reference op `op` (0 grey, 1 transpose, 2 gaussian, 3 fliplr, 4 rotate,
// 5 brightness, 6 colorize, 7 gamma) on a copy of `in`.  dims_io holds
// 2*ndims ints (shape then byte strides) and is updated in place, as the
// reference updates MPObjData.  Returns the output byte count, written to out.
long ref_run(int op, int type, int *ndims_io, int *dims_io, const void *in, long nbytes, double p0,
             double p1, double p2, void *out, long out_cap, int *type_out)
{
    MPObjData o;
    memset(&o, 0, sizeof(o));
    o.device_data = malloc(nbytes ? nbytes : 1);
    memcpy(o.device_data, in, nbytes);
    o.ndims = *ndims_io;
    o.dims = (int *)malloc(sizeof(int) * 2 * 4);
    memcpy(o.dims, dims_io, sizeof(int) * 2 * o.ndims);
    o.type = type;
    o.mem_loc = 0;
    o.stream = nullptr;
    o.nbytes = (size_t)nbytes;
    RotateArgs ra = {p0};
    GaussianArgs ga = {p0};
    BrightnessArgs ba = {p0};
    ColorizeArgs ca = {p0, p1, p2};
    GammaArgs gm = {p0, p1};
    switch (op) {
    case 0: mpimg_color_to_greyscale(&o, nullptr); break;
    case 1: mpimg_transpose(&o, nullptr); break;
    case 2: mpimg_gaussian(&o, &ga); break;
    case 3: mpimg_fliplr(&o, nullptr); break;
    case 4: mpimg_rotate(&o, &ra); break;
    case 5: mpimg_brightness(&o, &ba); break;
    case 6: mpimg_colorize(&o, &ca); break;
    case 7: mpimg_adjust_gamma(&o, &gm); break;
    default: break;
    }
    long n = (long)o.nbytes;
    if (n > out_cap) n = -1;
    else memcpy(out, o.device_data, n);
    *ndims_io = o.ndims;
    memcpy(dims_io, o.dims, sizeof(int) * 2 * o.ndims);
    *type_out = o.type;
    free(o.device_data);
    free(o.dims);
    return n;
}
}
