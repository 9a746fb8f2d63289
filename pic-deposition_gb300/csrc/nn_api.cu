// pic_nn_conv3x3: one convolution layer on host buffers (a stateless entry for
// checking the tensor-core kernels against the oracle; the warm-start training
// path in warmstart.cu keeps everything resident instead).
#include <vector>

#include "nn_conv.cuh"
#include "pic_internal.cuh"

using namespace picgb;

namespace {

struct DevBufs {
    std::vector<void*> p;
    ~DevBufs() {
        for (void* q : p) cudaFree(q);
    }
    template <typename T>
    T* alloc(size_t bytes, int* rc) {
        void* q = nullptr;
        const cudaError_t e = cudaMalloc(&q, bytes < 16 ? 16 : bytes);
        if (e != cudaSuccess) {
            *rc = cuda_fail(e, "cudaMalloc");
            return nullptr;
        }
        p.push_back(q);
        return static_cast<T*>(q);
    }
};

}  // namespace

extern "C" int pic_nn_conv3x3(int op, int batch, int H, int W, int cin, int cout, const uint16_t* x,
                              const float* weight, const float* bias, const uint16_t* aux, void* out) {
    if (!x || !out || batch <= 0 || H <= 0 || W <= 0) return fail(PIC_ERR_ARG, "pic_nn_conv3x3: bad argument");
    if ((cin != 16 && cin != 32) || (cout != 16 && cout != 32))
        return fail(PIC_ERR_ARG, "pic_nn_conv3x3: channels must be 16 or 32");
    if (op < 0 || op > 3) return fail(PIC_ERR_ARG, "pic_nn_conv3x3: unknown op");
    if ((op <= 1 && (!weight || !bias)) || (op == 2 && (!weight || !aux)) || (op == 3 && !aux))
        return fail(PIC_ERR_ARG, "pic_nn_conv3x3: missing operand");
    const size_t P = (size_t)batch * H * W;
    const int xin = op == 2 ? cout : cin;  // channels of x
    int rc = PIC_OK;
    DevBufs d;
    cudaStream_t s = nullptr;
    uint16_t* dx = d.alloc<uint16_t>(P * xin * 2, &rc);
    int* derr = d.alloc<int>(sizeof(int), &rc);
    if (rc) return rc;
    PIC_CUDA_TRY(cudaMemcpy(dx, x, P * xin * 2, cudaMemcpyHostToDevice));
    PIC_CUDA_TRY(cudaMemset(derr, 0, sizeof(int)));
    if (op == 3) {
        uint16_t* ddy = d.alloc<uint16_t>(P * cout * 2, &rc);
        const long long units = picnn::wgrad_units(batch, H, W);
        const int grid = picnn::wgrad_grid(units);
        const int upc = (int)((units + grid - 1) / grid);
        const int g2 = (int)((units + upc - 1) / upc);
        float* part = d.alloc<float>((size_t)g2 * picnn::wgrad_mpad(cin) * cout * 4, &rc);
        float* dwb = d.alloc<float>((size_t)(9 * cin * cout + cout) * 4, &rc);
        if (rc) return rc;
        PIC_CUDA_TRY(cudaMemcpy(ddy, aux, P * cout * 2, cudaMemcpyHostToDevice));
        picnn::WgradLaunch a{dx, ddy, part, batch, H, W, upc, derr};
        PIC_TRY(picnn::launch_wgrad(a, cin, cout, g2, s));
        PIC_TRY(picnn::reduce_wgrad(part, g2, cin, cout, dwb, dwb + 9 * cin * cout, s));
        PIC_CUDA_TRY(cudaDeviceSynchronize());
        PIC_CUDA_TRY(cudaMemcpy(out, dwb, (size_t)(9 * cin * cout + cout) * 4, cudaMemcpyDeviceToHost));
    } else {
        const int kcin = op == 2 ? cout : cin, kcout = op == 2 ? cin : cout;
        float* dw = d.alloc<float>((size_t)9 * cin * cout * 4, &rc);
        uint16_t* img = d.alloc<uint16_t>(picnn::wimg_bytes(cin, cout), &rc);
        float* db = d.alloc<float>((size_t)kcout * 4, &rc);
        uint16_t* dmask = op == 2 ? d.alloc<uint16_t>(P * kcout * 2, &rc) : nullptr;
        const size_t obytes = op == 1 ? P * 4 : P * kcout * 2;
        void* dout = d.alloc<uint8_t>(obytes, &rc);
        if (rc) return rc;
        PIC_CUDA_TRY(cudaMemcpy(dw, weight, (size_t)9 * cin * cout * 4, cudaMemcpyHostToDevice));
        if (op <= 1) PIC_CUDA_TRY(cudaMemcpy(db, bias, (size_t)kcout * 4, cudaMemcpyHostToDevice));
        if (op == 2) PIC_CUDA_TRY(cudaMemcpy(dmask, aux, P * kcout * 2, cudaMemcpyHostToDevice));
        PIC_TRY(picnn::build_weight_image(dw, cin, cout, op == 2 ? 1 : 0, img, s));
        picnn::ConvLaunch a{dx, img, db, dmask, dout, batch, H, W, 8, derr};
        const int epi = op == 0 ? picnn::EPI_BIAS_RELU : op == 1 ? picnn::EPI_BIAS_OUT : picnn::EPI_MASK;
        PIC_TRY(picnn::launch_conv(a, kcin, kcout, epi, s));
        PIC_CUDA_TRY(cudaDeviceSynchronize());
        PIC_CUDA_TRY(cudaMemcpy(out, dout, obytes, cudaMemcpyDeviceToHost));
    }
    int herr = 0;
    PIC_CUDA_TRY(cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost));
    if (herr) return fail(PIC_ERR_TIMEOUT, "pic_nn_conv3x3: a wait on the tensor cores timed out");
    return PIC_OK;
}
