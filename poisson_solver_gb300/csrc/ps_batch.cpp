// Batched solves: many independent problems (any grid, boundary conditions,
// components and output option each) run as five launches, one per pass,
// each launch covering the tiles of every problem (k_*_batch in ps_kernels_body.cuh).
// The five launches are captured once into a CUDA graph and replayed by every
// solve until the set of problems, their options or their pushed components
// change.
//
// Each problem keeps a ps::Solver for its state: the kernel build, the FFT
// plans and the device buffers. A solve reuses the solver's pass arguments
// (Solver::prepare) with the run-time kernel family, which covers every length.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "poisson_solver_gb300.h"
#include "ps_solver.hpp"

namespace ps {

#define PS_BCK(expr)                                                                                           \
    do {                                                                                                       \
        cudaError_t e_ = (expr);                                                                               \
        if (e_ != cudaSuccess) throw ps::Error(PS_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

struct Batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    int precision = PREC_FP64;
    std::vector<std::unique_ptr<Solver>> items;
    std::string last_error;

    // The executable: per pass, the arguments of every problem and the tile
    // list, in device memory, with the launch's block and shared-memory sizes.
    struct PassExec {
        DevBuf args, tiles;
        int ntiles = 0, nt = 0;
        size_t smem = 0;
        bool rader = false;  // a problem of the launch has a Rader plan
    };
    PassExec ex[5];
    // Launch shape of the x (passes 0 and 4), y (1 and 3) and z (2)
    // launches: the bound on a CTA's threads and the lines a CTA each problem
    // starts from (halved until it fits). ps_batch_autotune times the
    // choices; the defaults are the untuned shape.
    int cap[3] = {BATCH_MAX_THREADS, BATCH_MAX_THREADS, BATCH_MAX_THREADS};
    int start[3] = {16, 16, 16};
    // Plan variant (PV_* bits, FP32 only) of every problem's x, y and z
    // transforms; ps_batch_autotune times them too.
    int pv[3] = {0, 0, 0};
    std::vector<int> write_masks;  // outputs of each problem in the captured solve
    // Passes that a problem runs with its own kernel family instead of the
    // batched run-time launch (its usual choice, when that is not the
    // run-time family: power-of-two lengths in FP32), launched after the
    // batched launch of the pass with the problem's own arguments.
    std::vector<PassArgs> own_args;
    std::vector<std::array<PassChoice, 5>> own_choice;
    std::vector<int> routed[5];
    bool dirty = true;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;

    explicit Batch(int prec) : precision(prec)
    {
        if (prec == PREC_DF64) throw Error(PS_ERR_UNSUPPORTED, "double-float transforms are for single problems");
        if (prec != PREC_FP64 && prec != PREC_FP32) throw Error(PS_ERR_ARGUMENT, "precision must be FP64 or FP32");
        PS_BCK(cudaGetDevice(&device));
    }
    ~Batch() { release_graph(); }

    Solver &at(int i)
    {
        if (i < 0 || i >= (int)items.size()) throw Error(PS_ERR_ARGUMENT, "problem index out of range");
        return *items[i];
    }

    // A problem with the setup of an earlier one (another right-hand side of
    // the same problem) copies that problem's kernel octant instead of
    // building its own.
    int add(const int ncell[3], const int bc[3], const double dx[3], int reg)
    {
        auto s = std::make_unique<Solver>();
        s->stream = stream;
        s->precision = precision;
        for (const auto &o : items) {
            bool same = o->dims == 3 && o->reg == reg && o->kernel_family == s->kernel_family;
            for (int d = 0; d < 3 && same; ++d) same = o->n[d] == ncell[d] && o->bc[d] == bc[d] && o->dx[d] == dx[d];
            if (same) {
                s->kernel_from = o.get();
                break;
            }
        }
        s->setup3d(ncell, bc, dx, reg);
        s->kernel_from = nullptr;
        items.push_back(std::move(s));
        dirty = true;
        return (int)items.size() - 1;
    }

    void set_option(int i, int option, int value)
    {
        if (option == PS_OPT_PRECISION) throw Error(PS_ERR_ARGUMENT, "a batch has one precision, set at creation");
        at(i).set_option(option, value);
        dirty = true;
    }

    // kernel family of problem i: its kernel is rebuilt, as a new setup
    void set_kernel(int i, int family, double width)
    {
        at(i).set_kernel(family, width);
        dirty = true;
    }

    void push(int i, const double *const B[3], cudaMemcpyKind kind)
    {
        Solver &s = at(i);
        const int before = s.pushed;
        s.push(B, kind);
        if (s.pushed != before) dirty = true;
    }

    void pull(int i, double *const A[3], cudaMemcpyKind kind)
    {
        double *const none[3] = {nullptr, nullptr, nullptr};
        at(i).pull(A, none, kind);
    }

    void set_stream(cudaStream_t st)
    {
        stream = st;
        for (auto &s : items) s->stream = st;
    }

    void release_graph()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
    }

    // Lines per CTA of each problem in one batched pass. The launch's block
    // size nt is the largest of the problems' usual CTA sizes (capped at
    // BATCH_MAX_THREADS); each problem then takes the most lines (a power of
    // two) that fit nt threads and the largest usual shared-memory size, so
    // that its CTAs leave as few threads idle as the smem budget allows.
    template <typename SmemFn>
    static void choose_lines(const std::vector<int> &tpl, const SmemFn &smem, int max_lines, int max_threads,
                             int start_lines, std::vector<int> &B, int &nt, size_t &smem_max)
    {
        const size_t limit = (size_t)max_smem_per_block() - 2048;  // room for static shared data
        const int n = (int)tpl.size();
        B.assign(n, 1);
        nt = 0;
        size_t cap = 0;
        for (int p = 0; p < n; ++p) {
            int b = std::min(start_lines, max_lines);
            while (b > 1 && (b * tpl[p] > max_threads || smem(p, b) > limit)) b >>= 1;
            if (b * tpl[p] > max_threads || smem(p, b) > limit)
                throw Error(PS_ERR_UNSUPPORTED, "a transform of the batch is too long for one CTA");
            nt = std::max(nt, b * tpl[p]);
            cap = std::max(cap, smem(p, b));
        }
        smem_max = 0;
        for (int p = 0; p < n; ++p) {
            int b = 1;
            while (2 * b <= max_lines && 2 * b * tpl[p] <= nt && smem(p, 2 * b) <= cap) b *= 2;
            B[p] = b;
            smem_max = std::max(smem_max, smem(p, b));
        }
        nt = (nt + 31) / 32 * 32;
    }

    template <typename Args> static void upload(PassExec &e, const std::vector<Args> &args, const std::vector<BatchTile> &tiles)
    {
        e.ntiles = (int)tiles.size();
        e.rader = false;
        for (const BatchTile &t : tiles) e.rader = e.rader || args[t.p].plan.rader;
        if (args.empty() || tiles.empty()) return;
        e.args.ensure(args.size() * sizeof(Args));
        e.tiles.ensure(tiles.size() * sizeof(BatchTile));
        PS_BCK(cudaMemcpy(e.args.p, args.data(), args.size() * sizeof(Args), cudaMemcpyHostToDevice));
        PS_BCK(cudaMemcpy(e.tiles.p, tiles.data(), tiles.size() * sizeof(BatchTile), cudaMemcpyHostToDevice));
    }

    // Pass k of every problem on stream st: one batched launch over the
    // problems it covers, then the routed problems' own launches.
    cudaError_t launch(int k, cudaStream_t st)
    {
        const int prec = precision;
        const PassExec &e = ex[k];
        cudaError_t r;
        switch (k) {
        case 0:
            r = launch_xfwd_batch(prec, (const XFwdArgs *)e.args.p, (const BatchTile *)e.tiles.p, e.ntiles, e.nt,
                                  e.smem, e.rader, st);
            break;
        case 1:
        case 3:
            r = launch_col_batch(prec, k == 3, (const ColArgs *)e.args.p, (const BatchTile *)e.tiles.p, e.ntiles, e.nt,
                                 e.smem, e.rader, st);
            break;
        case 2:
            r = launch_z_batch(prec, (const ZArgs *)e.args.p, (const BatchTile *)e.tiles.p, e.ntiles, e.nt, e.smem,
                               e.rader, st);
            break;
        default:
            r = launch_xinv_batch(prec, (const XInvArgs *)e.args.p, (const BatchTile *)e.tiles.p, e.ntiles, e.nt,
                                  e.smem, e.rader, st);
        }
        if (r != cudaSuccess) return r;
        try {
            for (int p : routed[k]) items[p]->launch_on(k, own_choice[p][k], own_args[p], st);
        } catch (const Error &err) {
            throw Error(err.status, std::string("routed pass: ") + err.what());
        }
        return cudaSuccess;
    }

    // launches of one solve: the batched launches with tiles and the routed ones
    int launches_per_solve() const
    {
        int n = 0;
        for (int k = 0; k < 5; ++k) n += (ex[k].ntiles > 0) + (int)routed[k].size();
        return n;
    }

    void build()
    {
        prepare_passes();
        capture();
    }

    // The five passes' arguments and tile lists for the current launch
    // shapes, in device memory.
    void prepare_passes()
    {
        if (items.empty()) throw Error(PS_ERR_STATE, "the batch holds no problem");
        const int n = (int)items.size(), prec = precision;
        std::vector<PassArgs> pa(n);
        std::vector<const Plan *> plx(n), ply(n), plz(n);
        write_masks.assign(n, 0);
        own_choice.assign(n, {});
        for (auto &r : routed) r.clear();
        for (int p = 0; p < n; ++p) {
            Solver &s = *items[p];
            if (!s.pushed) throw Error(PS_ERR_STATE, "problem " + std::to_string(p) + ": solve called before push");
            const int out_mask = s.output_mask(s.pushed);
            const double *Bin[3];
            double *Aout[3];
            for (int c = 0; c < 3; ++c) {
                Bin[c] = (s.pushed >> c & 1) ? (const double *)s.fb[c].p : nullptr;
                Aout[c] = nullptr;
                if (out_mask >> c & 1) {
                    s.fa[c].ensure((size_t)s.n[0] * s.n[1] * s.n[2] * sizeof(double));
                    Aout[c] = (double *)s.fa[c].p;
                }
            }
            write_masks[p] = s.prepare(Bin, Aout, false, pa[p]);
            for (int k = 0; k < 5; ++k) {
                own_choice[p][k] = PassChoice{'r', 1};
                if (k >= 3 && !write_masks[p]) continue;
                const PassChoice c = s.pass_choice(k, pa[p]);
                if (c.fam != 'r') {
                    own_choice[p][k] = c;
                    routed[k].push_back(p);
                }
            }
            plx[p] = &s.plan(s.P[0], prec, 0, pv[0]);
            ply[p] = &s.plan(s.P[1], prec, 0, pv[1]);
            plz[p] = &s.plan(s.P[2], prec, e_max_z(prec), pv[2]);  // the z body's element budget
        }
        // launch shapes over the problems each batched launch covers (x: passes
        // 0 and 4, y: 1 and 3, z: 2)
        auto batched = [&](int p, int k) { return own_choice[p][k].fam == 'r'; };
        std::vector<int> gx, gy, gz;  // problems in the batched x, y and z launches
        for (int p = 0; p < n; ++p) {
            if (batched(p, 0) || (write_masks[p] && batched(p, 4))) gx.push_back(p);
            if (batched(p, 1) || (write_masks[p] && batched(p, 3))) gy.push_back(p);
            if (batched(p, 2)) gz.push_back(p);
        }
        std::vector<int> tx, ty, tz, Bgx, Bgy, Bgz, Bx(n, 1), By(n, 1), Bz(n, 1);
        for (int p : gx) tx.push_back(plx[p]->dev.tpl);
        for (int p : gy) ty.push_back(ply[p]->dev.tpl);
        for (int p : gz) tz.push_back(plz[p]->dev.tpl);
        choose_lines(tx, [&](int i, int B) { return smem_x(prec, plx[gx[i]]->dev, B); }, MAX_LINES, cap[0], start[0],
                     Bgx, ex[0].nt, ex[0].smem);
        choose_lines(ty, [&](int i, int B) { return smem_col(prec, ply[gy[i]]->dev, B); }, MAX_LINES, cap[1], start[1],
                     Bgy, ex[1].nt, ex[1].smem);
        choose_lines(
            tz,
            [&](int i, int B) {
                const int p = gz[i];
                return smem_z(prec, plz[p]->dev, B, std::max(pa[p].z.nin, pa[p].z.nout));
            },
            MAX_LINES, cap[2], start[2], Bgz, ex[2].nt, ex[2].smem);
        for (size_t i = 0; i < gx.size(); ++i) Bx[gx[i]] = Bgx[i];
        for (size_t i = 0; i < gy.size(); ++i) By[gy[i]] = Bgy[i];
        for (size_t i = 0; i < gz.size(); ++i) Bz[gz[i]] = Bgz[i];
        ex[3].nt = ex[1].nt;
        ex[3].smem = ex[1].smem;
        ex[4].nt = ex[0].nt;
        ex[4].smem = ex[0].smem;

        std::vector<XFwdArgs> ax(n);
        std::vector<ColArgs> ay(n), ayi(n);
        std::vector<ZArgs> az(n);
        std::vector<XInvArgs> axi(n);
        std::vector<BatchTile> t0, t1, t2, t3, t4;
        for (int p = 0; p < n; ++p) {
            const Solver &s = *items[p];
            ax[p] = pa[p].x;
            ax[p].plan = plx[p]->dev;
            ax[p].B = Bx[p];
            ay[p] = pa[p].y;
            ay[p].plan = ply[p]->dev;
            ay[p].B = By[p];
            az[p] = pa[p].z;
            az[p].plan = plz[p]->dev;
            az[p].B = Bz[p];
            ayi[p] = pa[p].yi;
            ayi[p].plan = ply[p]->dev;
            ayi[p].B = By[p];
            axi[p] = pa[p].xi;
            axi[p].plan = plx[p]->dev;
            axi[p].B = Bx[p];

            const long long lines = ((long long)s.n[1] * s.n[2] + 1) / 2;
            const int nbx = (int)((lines + Bx[p] - 1) / Bx[p]);
            if (batched(p, 0))
                for (int c = 0; c < ax[p].ncomp; ++c)
                    for (int b = 0; b < nbx; ++b) t0.push_back({p, b, c, 0});
            const int nby = (s.Mx + By[p] - 1) / By[p];
            if (batched(p, 1))
                for (int c = 0; c < ay[p].ncomp; ++c)
                    for (int z = 0; z < s.n[2]; ++z)
                        for (int b = 0; b < nby; ++b) t1.push_back({p, b, z, c});
            const int nbz = (s.Mx + Bz[p] - 1) / Bz[p];
            if (batched(p, 2))
                for (int ky = 0; ky < s.P[1]; ++ky)
                    for (int b = 0; b < nbz; ++b) t2.push_back({p, b, ky, 0});
            if (write_masks[p]) {
                if (batched(p, 3))
                    for (int c = 0; c < ayi[p].ncomp; ++c)
                        for (int z = 0; z < s.n[2]; ++z)
                            for (int b = 0; b < nby; ++b) t3.push_back({p, b, z, c});
                if (batched(p, 4))
                    for (int c = 0; c < axi[p].ncomp; ++c)
                        for (int b = 0; b < nbx; ++b) t4.push_back({p, b, c, 0});
            }
        }
        own_args = pa;
        PS_BCK(cudaStreamSynchronize(stream));  // kernel builds done before the arguments change hands
        upload(ex[0], ax, t0);
        upload(ex[1], ay, t1);
        upload(ex[2], az, t2);
        upload(ex[3], ayi, t3);
        upload(ex[4], axi, t4);
    }

    // Capture the five launches into the graph that solve() replays.
    void capture()
    {
        release_graph();
        cudaStream_t cs = stream;
        bool own = false;
        if (!cs) {
            // the legacy default stream cannot be captured: capture on a
            // private stream, replay on the batch's
            PS_BCK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
            own = true;
        }
        PS_BCK(cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed));
        cudaError_t e = cudaSuccess;
        std::string thrown;  // a routed launch's error: the capture still ends before it is reported
        int thrown_status = PS_OK;
        try {
            for (int k = 0; k < 5 && e == cudaSuccess; ++k) e = launch(k, cs);
        } catch (const Error &err) {
            thrown = err.what();
            thrown_status = err.status;
        }
        cudaGraph_t g = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(cs, &g);
        if (!thrown.empty()) {
            if (own) cudaStreamDestroy(cs);
            if (g) cudaGraphDestroy(g);
            throw Error(thrown_status, thrown);
        }
        if (own) cudaStreamDestroy(cs);
        if (e != cudaSuccess || ec != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            throw Error(PS_ERR_CUDA, std::string("batched launch capture: ") +
                                         cudaGetErrorString(e != cudaSuccess ? e : ec));
        }
        graph = g;
        PS_BCK(cudaGraphInstantiate(&exec, graph, 0));
        dirty = false;
    }

    // Time the plan variants (FP32) and then the launch shapes of each
    // axis's batched launches (the CTA size bound and the lines a CTA each
    // problem starts from) on the pushed problems and keep the fastest. The
    // per-line arithmetic does not depend on the shape; a plan variant
    // changes FP32 results at rounding level. Leaves the graph built.
    void autotune()
    {
        prepare_passes();  // buffers, plans and kernels of every problem
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        PS_BCK(cudaEventCreate(&e0));
        PS_BCK(cudaEventCreate(&e1));
        auto finish = [&] {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
        };
        try {
            static const int passes[3][2] = {{0, 4}, {1, 3}, {2, -1}};
            for (int ax = 0; ax < 3; ++ax) {
                // time the axis's launches in the current settings; < 0 if a
                // problem does not fit them
                auto time_axis = [&]() -> float {
                    try {
                        prepare_passes();
                    } catch (const Error &err) {
                        if (err.status == PS_ERR_UNSUPPORTED) return -1.f;
                        throw;
                    }
                    auto run_axis = [&] {
                        for (int k : passes[ax])
                            if (k >= 0) PS_BCK(launch(k, stream));
                    };
                    run_axis();  // warm-up (and the one-time attribute setup)
                    PS_BCK(cudaEventRecord(e0, stream));
                    const int reps = 3;
                    for (int r = 0; r < reps; ++r) run_axis();
                    PS_BCK(cudaEventRecord(e1, stream));
                    PS_BCK(cudaEventSynchronize(e1));
                    float ms = 0.f;
                    PS_BCK(cudaEventElapsedTime(&ms, e0, e1));
                    return ms;
                };
                float best_ms = -1.f;
                if (precision == PREC_FP32) {
                    // z bodies hold 8 elements a thread: no radix-cap variant
                    const int vmask = ax == 2 ? (PV_SMOOTH_M | PV_RADER) : (PV_HALF_RADIX | PV_SMOOTH_M | PV_RADER);
                    int best_pv = pv[ax];
                    for (int v = 0; v <= 7; ++v) {
                        if ((v & ~vmask) != 0) continue;
                        pv[ax] = v;
                        const float ms = time_axis();
                        if (ms >= 0.f && (best_ms < 0.f || ms < best_ms)) {
                            best_ms = ms;
                            best_pv = v;
                        }
                    }
                    pv[ax] = best_pv;
                }
                int best_cap = cap[ax], best_start = start[ax];
                best_ms = -1.f;
                for (int c : {64, 128, 256})
                    for (int l : {2, 4, 8, 16, 32}) {
                        cap[ax] = c;
                        start[ax] = l;
                        const float ms = time_axis();
                        if (ms >= 0.f && (best_ms < 0.f || ms < best_ms)) {
                            best_ms = ms;
                            best_cap = c;
                            best_start = l;
                        }
                    }
                cap[ax] = best_cap;
                start[ax] = best_start;
            }
        } catch (...) {
            finish();
            dirty = true;
            throw;
        }
        finish();
        build();
        dirty = false;
    }

    void solve()
    {
        if (dirty) build();
        PS_BCK(cudaGraphLaunch(exec, stream));
        for (size_t p = 0; p < items.size(); ++p) {
            items[p]->produced = write_masks[p];
            items[p]->rhs_ready = 0;
        }
    }

    long long tiles_per_solve() const
    {
        long long t = 0;
        for (const auto &e : ex) t += e.ntiles;
        return t;
    }
};

}  // namespace ps

struct ps_batch {
    std::unique_ptr<ps::Batch> b;
    std::string create_error;
};

namespace {

template <typename F> int bguarded(ps_batch *h, F &&f)
{
    if (!h || !h->b) return PS_ERR_ARGUMENT;
    ps::Batch &b = *h->b;
    try {
        ps::DeviceScope scope(b.device);
        f(b);
        b.last_error.clear();
        return PS_OK;
    } catch (const ps::Error &e) {
        b.last_error = e.what();
        return e.status;
    } catch (const std::bad_alloc &) {
        b.last_error = "host allocation failed";
        return PS_ERR_MEMORY;
    } catch (const std::exception &e) {
        b.last_error = e.what();
        return PS_ERR_CUDA;
    }
}

}  // namespace

extern "C" {

int ps_batch_create(ps_batch **out, int precision)
{
    if (!out) return PS_ERR_ARGUMENT;
    *out = nullptr;
    try {
        auto h = std::make_unique<ps_batch>();
        h->b = std::make_unique<ps::Batch>(precision);
        *out = h.release();
    } catch (const ps::Error &e) {
        return e.status;
    } catch (...) {
        return PS_ERR_MEMORY;
    }
    return PS_OK;
}

int ps_batch_destroy(ps_batch *h)
{
    if (!h) return PS_OK;
    if (h->b) {
        ps::DeviceScope scope(h->b->device);
        delete h;
    } else {
        delete h;
    }
    return PS_OK;
}

int ps_batch_add(ps_batch *h, const int ncell[3], const int bc[3], const double dx[3], int reg_order, int *index)
{
    if (!ncell || !bc || !dx) return PS_ERR_ARGUMENT;
    return bguarded(h, [&](ps::Batch &b) {
        const int i = b.add(ncell, bc, dx, reg_order);
        if (index) *index = i;
    });
}

int ps_batch_count(const ps_batch *h, int *count)
{
    if (!h || !h->b || !count) return PS_ERR_ARGUMENT;
    *count = (int)h->b->items.size();
    return PS_OK;
}

int ps_batch_set_option(ps_batch *h, int index, int option, int value)
{
    return bguarded(h, [&](ps::Batch &b) { b.set_option(index, option, value); });
}

int ps_batch_set_kernel(ps_batch *h, int index, int family, double width)
{
    return bguarded(h, [&](ps::Batch &b) { b.set_kernel(index, family, width); });
}

int ps_batch_push(ps_batch *h, int index, const double *bx, const double *by, const double *bz)
{
    return bguarded(h, [&](ps::Batch &b) {
        const double *B[3] = {bx, by, bz};
        b.push(index, B, cudaMemcpyHostToDevice);
    });
}

int ps_batch_push_device(ps_batch *h, int index, const double *bx, const double *by, const double *bz)
{
    return bguarded(h, [&](ps::Batch &b) {
        const double *B[3] = {bx, by, bz};
        b.push(index, B, cudaMemcpyDeviceToDevice);
    });
}

int ps_batch_solve(ps_batch *h)
{
    return bguarded(h, [&](ps::Batch &b) { b.solve(); });
}

int ps_batch_autotune(ps_batch *h)
{
    return bguarded(h, [&](ps::Batch &b) { b.autotune(); });
}

int ps_batch_get_tuning(const ps_batch *h, int axis, int *max_threads, int *start_lines, int *plan_variant)
{
    if (!h || !h->b || axis < 0 || axis > 2 || !max_threads || !start_lines || !plan_variant) return PS_ERR_ARGUMENT;
    const ps::Batch &b = *h->b;
    *max_threads = b.cap[axis];
    *start_lines = b.start[axis];
    *plan_variant = b.pv[axis];
    return PS_OK;
}

int ps_batch_set_tuning(ps_batch *h, int axis, int max_threads, int start_lines, int plan_variant)
{
    if (!h || !h->b || axis < 0 || axis > 2) return PS_ERR_ARGUMENT;
    if (max_threads < 32 || max_threads > ps::BATCH_MAX_THREADS || max_threads % 32 != 0) return PS_ERR_ARGUMENT;
    if (start_lines < 1 || start_lines > 64 || (start_lines & (start_lines - 1)) != 0) return PS_ERR_ARGUMENT;
    if (plan_variant < 0 || plan_variant > 7) return PS_ERR_ARGUMENT;
    ps::Batch &b = *h->b;
    b.cap[axis] = max_threads;
    b.start[axis] = start_lines;
    b.pv[axis] = plan_variant;
    b.dirty = true;  // the next solve rebuilds and recaptures
    return PS_OK;
}

int ps_batch_pull(ps_batch *h, int index, double *ax, double *ay, double *az)
{
    return bguarded(h, [&](ps::Batch &b) {
        double *A[3] = {ax, ay, az};
        b.pull(index, A, cudaMemcpyDeviceToHost);
    });
}

int ps_batch_pull_device(ps_batch *h, int index, double *ax, double *ay, double *az)
{
    return bguarded(h, [&](ps::Batch &b) {
        double *A[3] = {ax, ay, az};
        b.pull(index, A, cudaMemcpyDeviceToDevice);
    });
}

int ps_batch_set_stream(ps_batch *h, void *stream)
{
    return bguarded(h, [&](ps::Batch &b) { b.set_stream((cudaStream_t)stream); });
}

int ps_batch_synchronize(ps_batch *h)
{
    return bguarded(h, [&](ps::Batch &b) { PS_BCK(cudaStreamSynchronize(b.stream)); });
}

int ps_batch_get_info(const ps_batch *h, int what, double *value)
{
    if (!h || !h->b || !value) return PS_ERR_ARGUMENT;
    const ps::Batch &b = *h->b;
    switch (what) {
    case PS_BATCH_INFO_LAUNCHES_PER_SOLVE: *value = (double)b.launches_per_solve(); break;
    case PS_BATCH_INFO_TILES_PER_SOLVE: *value = (double)b.tiles_per_solve(); break;
    case PS_BATCH_INFO_POINTS: {
        double pts = 0;
        for (const auto &s : b.items) pts += (double)s->n[0] * s->n[1] * s->n[2];
        *value = pts;
        break;
    }
    case PS_BATCH_INFO_KERNEL_BUILDS: {
        int k = 0;
        for (const auto &s : b.items) k += s->kernel_builds;
        *value = (double)k;
        break;
    }
    default: return PS_ERR_ARGUMENT;
    }
    return PS_OK;
}

const char *ps_batch_last_error(const ps_batch *h)
{
    if (!h || !h->b) return "NULL batch handle";
    return h->b->last_error.c_str();
}

}  // extern "C"
