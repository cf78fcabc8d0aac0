// C ABI of the warm-start network (include/pfs.h: pfs_unet_*).
#include "kernels.h"
#include "pfs.h"
#include "unet.h"

using pfs::unet::Net;

extern "C" {

int pfs_unet_create(pfs_unet **out, long long max_pixels)
{
    if (!out || max_pixels <= 0 || max_pixels % (128 * 128))
        return pfs::record_error(PFS_ERR_INVALID_ARGUMENT, "max_pixels must be a positive multiple of 128*128");
    Net *n = nullptr;
    const int rc = pfs::unet::create(&n, (int)max_pixels);
    *out = reinterpret_cast<pfs_unet *>(n);
    return rc;
}

int pfs_unet_destroy(pfs_unet *u)
{
    pfs::unet::destroy(reinterpret_cast<Net *>(u));
    return PFS_OK;
}

long long pfs_unet_num_params(pfs_unet *u) { return u ? (long long)pfs::unet::num_params(reinterpret_cast<Net *>(u)) : 0; }

int pfs_unet_set_params(pfs_unet *u, const float *host)
{
    if (!u || !host) return pfs::record_error(PFS_ERR_INVALID_ARGUMENT, "null argument");
    return pfs::unet::set_params(reinterpret_cast<Net *>(u), host);
}

int pfs_unet_get_params(pfs_unet *u, float *host)
{
    if (!u || !host) return pfs::record_error(PFS_ERR_INVALID_ARGUMENT, "null argument");
    return pfs::unet::get_params(reinterpret_cast<Net *>(u), host);
}

int pfs_unet_get_grads(pfs_unet *u, float *host)
{
    if (!u || !host) return pfs::record_error(PFS_ERR_INVALID_ARGUMENT, "null argument");
    return pfs::unet::get_grads(reinterpret_cast<Net *>(u), host);
}

int pfs_unet_forward_backward(pfs_unet *u, const float *b, const float *p, int n, int h, int w, float *loss,
                              void *stream)
{
    if (!u || !b || !p || n <= 0) return pfs::record_error(PFS_ERR_INVALID_ARGUMENT, "bad arguments");
    return pfs::unet::forward_backward(reinterpret_cast<Net *>(u), b, p, n, h, w, loss, (cudaStream_t)stream);
}

int pfs_unet_adam_step(pfs_unet *u, float lr, void *stream)
{
    if (!u || !(lr > 0.0f)) return pfs::record_error(PFS_ERR_INVALID_ARGUMENT, "bad arguments");
    return pfs::unet::adam_step(reinterpret_cast<Net *>(u), lr, (cudaStream_t)stream);
}

int pfs_unet_predict(pfs_unet *u, const float *b, int ldb, float *p, int ldp, int h, int w, void *stream)
{
    if (!u || !b || !p || ldb < w || ldp < w) return pfs::record_error(PFS_ERR_INVALID_ARGUMENT, "bad arguments");
    return pfs::unet::predict(reinterpret_cast<Net *>(u), b, ldb, p, ldp, h, w, (cudaStream_t)stream);
}

int pfs_unet_predict_coarse(pfs_unet *u, const float *b, int ldb, float *p, int ldp, int h, int w, int coarsen,
                            void *stream)
{
    if (!u || !b || !p || ldb < w || ldp < w || coarsen < 1)
        return pfs::record_error(PFS_ERR_INVALID_ARGUMENT, "bad arguments");
    return pfs::unet::predict_coarse(reinterpret_cast<Net *>(u), b, ldb, p, ldp, h, w, coarsen, (cudaStream_t)stream);
}

}  // extern "C"
