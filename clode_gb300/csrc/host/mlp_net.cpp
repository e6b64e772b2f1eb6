// The surrogate network object behind the clode_mlp_* entry points: FP32
// master parameters with Adam moments, BF16 images of the tensor-core layer
// weights in both operand orders, the training data resident on the device,
// and one training step (14 kernels and a memset) captured as a CUDA graph
// and replayed.
//
// Parameter vector layout (FP32, row-major [in x out]):
//   W1 [2 x 256], b1 [256], W2 [256 x 256], b2 [256], W3 [256 x 256], b3 [256],
//   Wh [256 x H*K], bh [H*K]
// where the H heads predict the same K outputs (columns h*K .. h*K+K-1).
#include "common.hpp"
#include "mlp.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <random>
#include <vector>

using namespace clode;
using clode::mlp::bf16;
using clode::mlp::kWidth;

namespace {

struct Buf {
    void *p = nullptr;
    size_t bytes = 0;
    void reserve(size_t b)
    {
        if (b <= bytes && p)
            return;
        release();
        if (!b)
            return;
        if (cudaMalloc(&p, b) != cudaSuccess) {
            p = nullptr;
            bytes = 0;
            cudaGetLastError();
            fail(CLODE_ERR_OUT_OF_MEMORY, "cannot allocate %.3f GB on the device", b / 1e9);
        }
        bytes = b;
    }
    void release()
    {
        if (p)
            cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <typename T>
    T *as() const { return (T *)p; }
};

thread_local std::string g_mlp_error;

}  // namespace

struct clode_mlp {
    int K = 4, H = 4, HK = 16;
    int device = 0, sms = 1;
    cudaStream_t stream = nullptr;
    // offsets into the parameter vector
    size_t oW1, ob1, oW2, ob2, oW3, ob3, oWh, obh, n_params;
    Buf params, grads, m1, m2;
    Buf wf2, wb2, wf3, wb3, wfh, wbh;  // BF16 operand images (forward / backward order)
    mlp::WeightImages images[3];
    // batch work buffers (capacity cap rows, whole 128-row tiles)
    int cap = 0;
    Buf xb, yb, h1, c1, h2, h3, out, dzo, dz3, dz2, dz1;
    // training data and counters
    Buf xs, ys, counters, loss_hist;  // counters: [0] step, [1] cursor, [2] error flag, [3] loss, [4] history index
    long long data_rows = 0;
    // prediction results
    Buf pred_mean, pred_spread, pred_scaled;
    long long pred_rows = 0;
    Buf thr, flags;
    double train_ms = 0, predict_ms = 0;
    cudaGraphExec_t graph = nullptr;
    // what the captured training step baked in
    struct GraphKey {
        int batch = 0;
        float lr = 0;
        long long rows = 0;
        const void *xs = nullptr, *ys = nullptr, *hist = nullptr;
        bool operator==(const GraphKey &o) const
        {
            return batch == o.batch && lr == o.lr && rows == o.rows && xs == o.xs && ys == o.ys && hist == o.hist;
        }
    } graph_key;

    ~clode_mlp()
    {
        cudaSetDevice(device);
        if (graph)
            cudaGraphExecDestroy(graph);
        for (Buf *b : {&params, &grads, &m1, &m2, &wf2, &wb2, &wf3, &wb3, &wfh, &wbh, &xb, &yb, &h1, &c1, &h2, &h3,
                       &out, &dzo, &dz3, &dz2, &dz1, &xs, &ys, &counters, &loss_hist, &pred_mean, &pred_spread, &pred_scaled, &thr,
                       &flags})
            b->release();
        if (stream)
            cudaStreamDestroy(stream);
    }

    float *P(size_t off) const { return params.as<float>() + off; }
    float *G(size_t off) const { return grads.as<float>() + off; }
    int *step_ctr() const { return counters.as<int>(); }
    int *cursor_ctr() const { return counters.as<int>() + 1; }
    int *err_flag() const { return counters.as<int>() + 2; }
    float *loss_acc() const { return (float *)(counters.as<int>() + 3); }
    int *hist_index() const { return counters.as<int>() + 4; }

    void init(int k, int h, int dev, unsigned long long seed)
    {
        K = k;
        H = h;
        HK = k * h;
        if (HK != 16 && HK != 32 && HK != 64)
            fail(CLODE_ERR_INVALID_ARGUMENT, "heads x outputs must be 16, 32 or 64 (got %d x %d)", h, k);
        device = dev;
        use_device(device);
        check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "SM count");
        check_cuda(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "stream");
        oW1 = 0;
        ob1 = oW1 + 2 * kWidth;
        oW2 = ob1 + kWidth;
        ob2 = oW2 + (size_t)kWidth * kWidth;
        oW3 = ob2 + kWidth;
        ob3 = oW3 + (size_t)kWidth * kWidth;
        oWh = ob3 + kWidth;
        obh = oWh + (size_t)kWidth * HK;
        n_params = obh + HK;
        params.reserve(n_params * 4);
        grads.reserve(n_params * 4);
        m1.reserve(n_params * 4);
        m2.reserve(n_params * 4);
        for (Buf *b : {&wf2, &wb2, &wf3, &wb3})
            b->reserve((size_t)kWidth * kWidth * 2);
        wfh.reserve((size_t)kWidth * HK * 2);
        wbh.reserve((size_t)kWidth * HK * 2);
        images[0] = {oW2, kWidth, kWidth, wf2.as<bf16>(), wb2.as<bf16>()};
        images[1] = {oW3, kWidth, kWidth, wf3.as<bf16>(), wb3.as<bf16>()};
        images[2] = {oWh, kWidth, HK, wfh.as<bf16>(), wbh.as<bf16>()};
        counters.reserve(64);
        check_cuda(cudaMemset(counters.p, 0, 64), "counters");
        // first layer: frequencies U(-kInputScale, kInputScale) and phases
        // U(-pi, pi) of the sine encoding; He-uniform ReLU layers; uniform
        // 1/sqrt(fan_in) heads; zero biases elsewhere
        std::mt19937_64 gen(seed);
        std::vector<float> w(n_params, 0.0f);
        auto fill = [&](size_t off, size_t n, double a) {
            std::uniform_real_distribution<double> d(-a, a);
            for (size_t i = 0; i < n; ++i)
                w[off + i] = (float)d(gen);
        };
        fill(oW1, 2 * kWidth, kInputScale);
        fill(ob1, kWidth, 3.14159265358979);
        fill(oW2, (size_t)kWidth * kWidth, std::sqrt(6.0 / kWidth));
        fill(oW3, (size_t)kWidth * kWidth, std::sqrt(6.0 / kWidth));
        fill(oWh, (size_t)kWidth * HK, std::sqrt(1.0 / kWidth));
        set_params(w.data());
    }

    static constexpr double kInputScale = 20.0;

    // upload FP32 parameters, rebuild the BF16 images, reset Adam
    void set_params(const float *w)
    {
        use_device(device);
        check_cuda(cudaMemcpy(params.p, w, n_params * 4, cudaMemcpyHostToDevice), "parameters upload");
        check_cuda(cudaMemset(m1.p, 0, n_params * 4), "moments");
        check_cuda(cudaMemset(m2.p, 0, n_params * 4), "moments");
        mlp::write_images(params.as<float>(), images, 3, stream);
        int zero = 0;
        check_cuda(cudaMemcpyAsync(step_ctr(), &zero, sizeof zero, cudaMemcpyHostToDevice, stream), "counters");
        check_cuda(cudaStreamSynchronize(stream), "parameters upload");
    }

    void ensure_capacity(int rows)
    {
        if (rows <= cap)
            return;
        cap = rows;
        const size_t tr = (size_t)mlp::tiled_rows(rows);
        xb.reserve(tr * 2 * 4);
        yb.reserve(tr * K * 4);
        for (Buf *b : {&h1, &c1, &h2, &h3, &dz3, &dz2, &dz1})
            b->reserve(tr * kWidth * 2);
        out.reserve(tr * HK * 4);
        dzo.reserve(tr * HK * 2);
        if (graph) {
            cudaGraphExecDestroy(graph);
            graph = nullptr;
        }
    }

    // forward on the rows in xb -> h1 (sine), h2, h3, out
    void forward(int rows)
    {
        mlp::input_layer(xb.as<float>(), rows, P(oW1), P(ob1), h1.as<bf16>(), c1.as<bf16>(), stream);
        mlp::linear_relu(h1.as<bf16>(), rows, wf2.as<bf16>(), P(ob2), h2.as<bf16>(), err_flag(), sms, stream);
        mlp::linear_relu(h2.as<bf16>(), rows, wf3.as<bf16>(), P(ob3), h3.as<bf16>(), err_flag(), sms, stream);
        mlp::linear_heads(h3.as<bf16>(), rows, wfh.as<bf16>(), P(obh), out.as<float>(), HK, err_flag(), sms, stream);
    }

    // loss and gradients of the batch in xb / yb into grads (the loss
    // accumulator must be zero on entry)
    void backward(int rows)
    {
        check_cuda(cudaMemsetAsync(grads.p, 0, n_params * 4, stream), "gradient reset");
        mlp::mse(out.as<float>(), yb.as<float>(), rows, H, K, dzo.as<bf16>(), loss_acc(), stream);
        mlp::weight_grad(h3.as<bf16>(), dzo.as<bf16>(), HK, rows, G(oWh), G(obh), err_flag(), stream);
        mlp::linear_back_heads(dzo.as<bf16>(), rows, wbh.as<bf16>(), h3.as<bf16>(), dz3.as<bf16>(), HK, err_flag(),
                               sms, stream);
        mlp::weight_grad(h2.as<bf16>(), dz3.as<bf16>(), kWidth, rows, G(oW3), G(ob3), err_flag(), stream);
        mlp::linear_back_relu(dz3.as<bf16>(), rows, wb3.as<bf16>(), h2.as<bf16>(), dz2.as<bf16>(), err_flag(), sms,
                              stream);
        mlp::weight_grad(h1.as<bf16>(), dz2.as<bf16>(), kWidth, rows, G(oW2), G(ob2), err_flag(), stream);
        mlp::linear_back_mul(dz2.as<bf16>(), rows, wb2.as<bf16>(), c1.as<bf16>(), dz1.as<bf16>(), err_flag(), sms,
                             stream);
        mlp::weight_grad_input(xb.as<float>(), dz1.as<bf16>(), rows, G(oW1), G(ob1), stream);
    }

    void check_error_flag()
    {
        int e = 0;
        check_cuda(cudaMemcpy(&e, err_flag(), sizeof e, cudaMemcpyDeviceToHost), "error flag");
        if (e)
            fail(CLODE_ERR_CUDA, "a tensor-core layer timed out waiting for a copy or its MMA group (results invalid)");
    }

    void gradients(const float *x, const float *y, int rows, float *g_out, float *loss)
    {
        use_device(device);
        ensure_capacity(rows);
        check_cuda(cudaMemcpyAsync(xb.p, x, (size_t)rows * 2 * 4, cudaMemcpyHostToDevice, stream), "H2D");
        check_cuda(cudaMemcpyAsync(yb.p, y, (size_t)rows * K * 4, cudaMemcpyHostToDevice, stream), "H2D");
        check_cuda(cudaMemsetAsync(loss_acc(), 0, 4, stream), "loss reset");
        forward(rows);
        backward(rows);
        check_cuda(cudaMemcpyAsync(g_out, grads.p, n_params * 4, cudaMemcpyDeviceToHost, stream), "D2H");
        check_cuda(cudaMemcpyAsync(loss, loss_acc(), 4, cudaMemcpyDeviceToHost, stream), "D2H");
        check_cuda(cudaStreamSynchronize(stream), "gradients");
        check_error_flag();
    }

    void train(const float *x, const float *y, long long n, int steps, int batch, float lr, unsigned long long seed,
               float *loss_history)
    {
        if (n < 1 || steps < 0 || batch < 1)
            fail(CLODE_ERR_INVALID_ARGUMENT, "train: need n >= 1, steps >= 0, batch >= 1");
        if (n > 0x7FFFFFFFLL)
            fail(CLODE_ERR_INVALID_ARGUMENT, "train: at most 2^31 - 1 rows");
        use_device(device);
        // one shuffled copy of the data on the device; batches walk through it
        std::vector<long long> perm((size_t)n);
        for (long long i = 0; i < n; ++i)
            perm[(size_t)i] = i;
        std::mt19937_64 gen(seed);
        std::shuffle(perm.begin(), perm.end(), gen);
        std::vector<float> xsh((size_t)n * 2), ysh((size_t)n * K);
        for (long long i = 0; i < n; ++i) {
            long long r = perm[(size_t)i];
            xsh[2 * i] = x[2 * r];
            xsh[2 * i + 1] = x[2 * r + 1];
            for (int k = 0; k < K; ++k)
                ysh[(size_t)i * K + k] = y[(size_t)r * K + k];
        }
        xs.reserve((size_t)n * 2 * 4);
        ys.reserve((size_t)n * K * 4);
        check_cuda(cudaMemcpy(xs.p, xsh.data(), xsh.size() * 4, cudaMemcpyHostToDevice), "training data upload");
        check_cuda(cudaMemcpy(ys.p, ysh.data(), ysh.size() * 4, cudaMemcpyHostToDevice), "training data upload");
        data_rows = n;
        ensure_capacity(batch);
        loss_hist.reserve((size_t)(steps > 0 ? steps : 1) * 4);
        check_cuda(cudaMemsetAsync(cursor_ctr(), 0, sizeof(int), stream), "cursor");
        check_cuda(cudaMemsetAsync(hist_index(), 0, sizeof(int), stream), "history index");

        auto one_step = [&]() {
            mlp::gather_batch(xs.as<float>(), ys.as<float>(), (int)n, K, batch, cursor_ctr(), xb.as<float>(),
                              yb.as<float>(), step_ctr(), loss_acc(), stream);
            forward(batch);
            backward(batch);
            mlp::adam_all(params.as<float>(), grads.as<float>(), m1.as<float>(), m2.as<float>(), n_params, lr,
                          step_ctr(), images, 3, cursor_ctr(), loss_acc(), loss_hist.as<float>(), hist_index(),
                          stream);
        };
        auto t0 = std::chrono::steady_clock::now();
        if (steps > 0) {
            // first step eagerly (sets kernel attributes), the rest as a replayed graph
            one_step();
            if (steps > 1) {
                GraphKey key;
                key.batch = batch;
                key.lr = lr;
                key.rows = n;
                key.xs = xs.p;
                key.ys = ys.p;
                key.hist = loss_hist.p;
                if (!graph || !(graph_key == key)) {
                    if (graph) {
                        cudaGraphExecDestroy(graph);
                        graph = nullptr;
                    }
                    cudaGraph_t g;
                    check_cuda(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "graph capture");
                    one_step();
                    check_cuda(cudaStreamEndCapture(stream, &g), "graph capture");
                    check_cuda(cudaGraphInstantiate(&graph, g, 0), "graph instantiate");
                    cudaGraphDestroy(g);
                    graph_key = key;
                }
                for (int s = 1; s < steps; ++s) {
                    check_cuda(cudaGraphLaunch(graph, stream), "graph launch");
                    count_launch();
                }
            }
        }
        check_cuda(cudaStreamSynchronize(stream), "training");
        train_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        check_error_flag();
        if (loss_history && steps > 0)
            check_cuda(cudaMemcpy(loss_history, loss_hist.p, (size_t)steps * 4, cudaMemcpyDeviceToHost), "D2H");
    }

    void predict(const float *x, long long n, float *mean, float *spread, float *heads)
    {
        use_device(device);
        const int chunk = 1 << 22;
        ensure_capacity((int)std::min<long long>(n, chunk));
        pred_mean.reserve((size_t)std::max<long long>(n, 1) * K * 4);
        pred_spread.reserve((size_t)std::max<long long>(n, 1) * K * 4);
        pred_rows = n;
        auto t0 = std::chrono::steady_clock::now();
        for (long long r0 = 0; r0 < n; r0 += chunk) {
            int rows = (int)std::min<long long>(chunk, n - r0);
            check_cuda(cudaMemcpyAsync(xb.p, x + 2 * r0, (size_t)rows * 2 * 4, cudaMemcpyHostToDevice, stream), "H2D");
            forward(rows);
            mlp::head_stats(out.as<float>(), rows, H, K, pred_mean.as<float>() + r0 * K,
                            pred_spread.as<float>() + r0 * K, stream);
            if (heads)
                check_cuda(cudaMemcpyAsync(heads + r0 * HK, out.p, (size_t)rows * HK * 4, cudaMemcpyDeviceToHost,
                                           stream),
                           "D2H");
        }
        if (mean)
            check_cuda(cudaMemcpyAsync(mean, pred_mean.p, (size_t)n * K * 4, cudaMemcpyDeviceToHost, stream), "D2H");
        if (spread)
            check_cuda(cudaMemcpyAsync(spread, pred_spread.p, (size_t)n * K * 4, cudaMemcpyDeviceToHost, stream),
                       "D2H");
        check_cuda(cudaStreamSynchronize(stream), "prediction");
        predict_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        check_error_flag();
    }

    void predict_grid(int nx, int ny, const float *out_scale, const float *out_offset, float *out_h)
    {
        use_device(device);
        const long long n = (long long)nx * ny;
        const int chunk = 1 << 22;
        ensure_capacity((int)std::min<long long>(n, chunk));
        pred_mean.reserve((size_t)std::max<long long>(n, 1) * K * 4);
        pred_spread.reserve((size_t)std::max<long long>(n, 1) * K * 4);
        pred_scaled.reserve((size_t)std::max<long long>(n, 1) * K * 4);
        thr.reserve((size_t)2 * K * 4);
        std::vector<float> so(2 * (size_t)K);
        for (int k = 0; k < K; ++k) {
            so[k] = out_scale ? out_scale[k] : 1.0f;
            so[K + k] = out_offset ? out_offset[k] : 0.0f;
        }
        pred_rows = n;
        auto t0 = std::chrono::steady_clock::now();
        check_cuda(cudaMemcpyAsync(thr.p, so.data(), so.size() * 4, cudaMemcpyHostToDevice, stream), "H2D");
        for (long long r0 = 0; r0 < n; r0 += chunk) {
            int rows = (int)std::min<long long>(chunk, n - r0);
            mlp::grid_inputs(nx, ny, r0, rows, xb.as<float>(), stream);
            forward(rows);
            mlp::head_stats(out.as<float>(), rows, H, K, pred_mean.as<float>() + r0 * K,
                            pred_spread.as<float>() + r0 * K, stream, thr.as<float>(), thr.as<float>() + K,
                            pred_scaled.as<float>() + r0 * K);
        }
        check_cuda(cudaMemcpyAsync(out_h, pred_scaled.p, (size_t)n * K * 4, cudaMemcpyDeviceToHost, stream), "D2H");
        check_cuda(cudaStreamSynchronize(stream), "grid prediction");
        predict_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        check_error_flag();
    }

    void screen(int nx, int ny, const float *spread_thr, const float *jump_thr, int *flags_out)
    {
        if ((long long)nx * ny != pred_rows)
            fail(CLODE_ERR_INVALID_ARGUMENT, "grid %d x %d does not match the last prediction (%lld points)", nx, ny,
                 pred_rows);
        use_device(device);
        thr.reserve((size_t)2 * K * 4);
        check_cuda(cudaMemcpy(thr.p, spread_thr, (size_t)K * 4, cudaMemcpyHostToDevice), "H2D");
        check_cuda(cudaMemcpy(thr.as<float>() + K, jump_thr, (size_t)K * 4, cudaMemcpyHostToDevice), "H2D");
        flags.reserve((size_t)pred_rows * 4);
        mlp::screen_grid(pred_mean.as<float>(), pred_spread.as<float>(), nx, ny, K, thr.as<float>(),
                         thr.as<float>() + K, flags.as<int>(), stream);
        check_cuda(cudaMemcpyAsync(flags_out, flags.p, (size_t)pred_rows * 4, cudaMemcpyDeviceToHost, stream), "D2H");
        check_cuda(cudaStreamSynchronize(stream), "screening");
    }
};

namespace {
template <typename F>
int mlp_guard(F &&f)
{
    try {
        f();
        g_mlp_error.clear();
        set_last_error_message("");
        return CLODE_OK;
    } catch (const Error &e) {
        set_last_error_message(e.what());
        return e.code;
    } catch (const std::bad_alloc &) {
        set_last_error_message("host allocation failed");
        return CLODE_ERR_OUT_OF_MEMORY;
    } catch (const std::exception &e) {
        set_last_error_message(e.what());
        return CLODE_ERR_INTERNAL;
    }
}
}  // namespace

extern "C" {

int clode_mlp_create(int n_outputs, int n_heads, int device, unsigned long long seed, clode_mlp **out)
{
    return mlp_guard([&] {
        if (!out)
            fail(CLODE_ERR_INVALID_ARGUMENT, "out must not be NULL");
        std::unique_ptr<clode_mlp> net(new clode_mlp());
        net->init(n_outputs, n_heads, device, seed);
        *out = net.release();
    });
}

int clode_mlp_destroy(clode_mlp *net)
{
    return mlp_guard([&] { delete net; });
}

int clode_mlp_param_count(clode_mlp *net, size_t *n)
{
    return mlp_guard([&] {
        if (!net || !n)
            fail(CLODE_ERR_INVALID_ARGUMENT, "NULL argument");
        *n = net->n_params;
    });
}

int clode_mlp_get_params(clode_mlp *net, float *out, size_t n)
{
    return mlp_guard([&] {
        if (!net || !out || n < net->n_params)
            fail(CLODE_ERR_INVALID_ARGUMENT, "need %zu floats", net ? net->n_params : (size_t)0);
        use_device(net->device);
        check_cuda(cudaMemcpy(out, net->params.p, net->n_params * 4, cudaMemcpyDeviceToHost), "D2H");
    });
}

int clode_mlp_set_params(clode_mlp *net, const float *in, size_t n)
{
    return mlp_guard([&] {
        if (!net || !in || n != net->n_params)
            fail(CLODE_ERR_INVALID_ARGUMENT, "need exactly %zu floats", net ? net->n_params : (size_t)0);
        net->set_params(in);
    });
}

int clode_mlp_gradients(clode_mlp *net, const float *x, const float *y, int n, float *grads, size_t n_grads,
                        float *loss)
{
    return mlp_guard([&] {
        if (!net || !x || !y || !grads || !loss || n < 1 || n_grads < net->n_params)
            fail(CLODE_ERR_INVALID_ARGUMENT, "invalid arguments");
        net->gradients(x, y, n, grads, loss);
    });
}

int clode_mlp_train(clode_mlp *net, const float *x, const float *y, long long n, int steps, int batch, float lr,
                    unsigned long long seed, float *loss_history)
{
    return mlp_guard([&] {
        if (!net || !x || !y)
            fail(CLODE_ERR_INVALID_ARGUMENT, "invalid arguments");
        net->train(x, y, n, steps, batch, lr, seed, loss_history);
    });
}

int clode_mlp_predict(clode_mlp *net, const float *x, long long n, float *mean, float *spread, float *heads)
{
    return mlp_guard([&] {
        if (!net || !x || n < 0)
            fail(CLODE_ERR_INVALID_ARGUMENT, "invalid arguments");
        net->predict(x, n, mean, spread, heads);
    });
}

int clode_mlp_predict_grid(clode_mlp *net, int nx, int ny, const float *out_scale, const float *out_offset,
                           float *out)
{
    return mlp_guard([&] {
        if (!net || !out || nx < 1 || ny < 1)
            fail(CLODE_ERR_INVALID_ARGUMENT, "invalid arguments");
        net->predict_grid(nx, ny, out_scale, out_offset, out);
    });
}

int clode_mlp_screen(clode_mlp *net, int nx, int ny, const float *spread_thr, const float *jump_thr, int *flags)
{
    return mlp_guard([&] {
        if (!net || !spread_thr || !jump_thr || !flags || nx < 1 || ny < 1)
            fail(CLODE_ERR_INVALID_ARGUMENT, "invalid arguments");
        net->screen(nx, ny, spread_thr, jump_thr, flags);
    });
}

int clode_mlp_timings(clode_mlp *net, double *train_ms, double *predict_ms)
{
    return mlp_guard([&] {
        if (!net)
            fail(CLODE_ERR_INVALID_ARGUMENT, "NULL net");
        if (train_ms)
            *train_ms = net->train_ms;
        if (predict_ms)
            *predict_ms = net->predict_ms;
    });
}

}  // extern "C"
