// extern "C" face of the learned preconditioner's network (include/m3d_gb300.h,
// "Learned preconditioner network"): host arrays in and out, so that the
// tensor-core kernels can be checked against a CPU restatement.  The solver
// uses the same class directly (solver.cu).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstring>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "m3d_gb300.h"
#include "cuda/learned.cuh"

struct m3d_cnn {
    m3d::learn::Cnn* net = nullptr;
    std::string err;
};

namespace {

template <class F>
int cnn_guarded(m3d_cnn* h, F&& f) {
    if (!h || !h->net) return M3D_ERR_ARG;
    try {
        f(*h->net);
        return M3D_OK;
    } catch (const std::bad_alloc&) {
        cudaGetLastError();
        h->err = "allocation failed";
        return M3D_ERR_OOM;
    } catch (const std::invalid_argument& e) {
        h->err = e.what();
        return M3D_ERR_ARG;
    } catch (const std::exception& e) {
        h->err = e.what();
        return M3D_ERR_CUDA;
    }
}

// host FP32 [G][c] -> device BF16 [G][32] input of the network
void upload_input(m3d::learn::Cnn& net, const float* x, long long G, int c) {
    std::vector<__nv_bfloat16> h((size_t)G * m3d::learn::kCh, __float2bfloat16(0.0f));
    for (long long g = 0; g < G; ++g)
        for (int k = 0; k < c; ++k) h[(size_t)g * m3d::learn::kCh + k] = __float2bfloat16(x[(size_t)g * c + k]);
    if (cudaMemcpyAsync(net.input(), h.data(), h.size() * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice,
                        net.stream()) != cudaSuccess ||
        cudaStreamSynchronize(net.stream()) != cudaSuccess) {
        cudaGetLastError();
        throw std::runtime_error("cnn: input upload failed");
    }
}

void check_flag(m3d::learn::Cnn& net) {
    if (net.error_flag()) throw std::runtime_error("cnn: a tensor-core kernel's barrier wait timed out");
}

template <class T>
struct DevBuf {
    T* p = nullptr;
    explicit DevBuf(size_t n) {
        if (cudaMalloc(&p, (n ? n : 1) * sizeof(T)) != cudaSuccess) {
            cudaGetLastError();
            throw std::bad_alloc();
        }
    }
    ~DevBuf() { if (p) cudaFree(p); }
};

}  // namespace

extern "C" int m3d_cnn_create(int device, int layers, int c_in, int hidden, int c_out, unsigned seed, m3d_cnn** out) {
    if (!out) return M3D_ERR_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return M3D_ERR_NO_DEVICE;
    }
    try {
        auto* h = new m3d_cnn();
        h->net = new m3d::learn::Cnn(device, layers, c_in, hidden, c_out, seed);
        *out = h;
        return M3D_OK;
    } catch (const std::invalid_argument&) {
        return M3D_ERR_ARG;
    } catch (const std::bad_alloc&) {
        cudaGetLastError();
        return M3D_ERR_OOM;
    } catch (...) {
        cudaGetLastError();
        return M3D_ERR_CUDA;
    }
}

extern "C" void m3d_cnn_destroy(m3d_cnn* h) {
    if (!h) return;
    delete h->net;
    delete h;
}

extern "C" const char* m3d_cnn_last_error(const m3d_cnn* h) { return h ? h->err.c_str() : "null handle"; }

extern "C" int m3d_cnn_get_weights(m3d_cnn* h, float* w, float* b) {
    if (!w || !b) return M3D_ERR_ARG;
    return cnn_guarded(h, [&](m3d::learn::Cnn& net) { net.get_weights(w, b); });
}

extern "C" int m3d_cnn_set_weights(m3d_cnn* h, const float* w, const float* b) {
    if (!w || !b) return M3D_ERR_ARG;
    return cnn_guarded(h, [&](m3d::learn::Cnn& net) { net.set_weights(w, b); });
}

extern "C" int m3d_cnn_forward(m3d_cnn* h, const float* x, int n, int D, int H, int W, float* y) {
    if (!x || !y || n < 1) return M3D_ERR_ARG;
    return cnn_guarded(h, [&](m3d::learn::Cnn& net) {
        net.ensure(n, D, H, W);
        const long long G = (long long)n * D * H * W;
        upload_input(net, x, G, net.c_in());
        const float* o = net.forward(n);
        check_flag(net);
        if (cudaMemcpy(y, o, (size_t)G * net.c_out() * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) {
            cudaGetLastError();
            throw std::runtime_error("cnn: output copy failed");
        }
    });
}

extern "C" int m3d_cnn_backward(m3d_cnn* h, const float* x, const float* dy, int n, int D, int H, int W, float* dw,
                                float* db, float* dx) {
    if (!x || !dy || !dw || !db || n < 1) return M3D_ERR_ARG;
    return cnn_guarded(h, [&](m3d::learn::Cnn& net) {
        net.ensure(n, D, H, W);
        const long long G = (long long)n * D * H * W;
        upload_input(net, x, G, net.c_in());
        net.forward(n);
        DevBuf<float> d_dy((size_t)G * net.c_out());
        DevBuf<float> d_dx((size_t)G * m3d::learn::kCh);
        if (cudaMemcpy(d_dy.p, dy, (size_t)G * net.c_out() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
            throw std::runtime_error("cnn: upload failed");
        net.backward(n, d_dy.p, dx ? d_dx.p : nullptr);
        check_flag(net);
        net.get_grads(dw, db);
        if (dx) {
            std::vector<float> t((size_t)G * m3d::learn::kCh);
            if (cudaMemcpy(t.data(), d_dx.p, t.size() * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
                throw std::runtime_error("cnn: copy failed");
            for (long long g = 0; g < G; ++g)
                for (int k = 0; k < net.c_in(); ++k) dx[(size_t)g * net.c_in() + k] = t[(size_t)g * m3d::learn::kCh + k];
        }
    });
}

extern "C" int m3d_cnn_train_step(m3d_cnn* h, const float* x, const float* target, int n, int D, int H, int W,
                                  float lr, double* loss) {
    if (!x || !target || n < 1 || !(lr > 0.0f)) return M3D_ERR_ARG;
    return cnn_guarded(h, [&](m3d::learn::Cnn& net) {
        net.ensure(n, D, H, W);
        const long long G = (long long)n * D * H * W;
        upload_input(net, x, G, net.c_in());
        DevBuf<float> d_t((size_t)G * net.c_out());
        if (cudaMemcpy(d_t.p, target, (size_t)G * net.c_out() * sizeof(float), cudaMemcpyHostToDevice) !=
            cudaSuccess)
            throw std::runtime_error("cnn: upload failed");
        net.forward(n);
        const double l = net.loss_backward(n, d_t.p);
        net.adam_step(lr);
        check_flag(net);
        if (loss) *loss = l;
    });
}
