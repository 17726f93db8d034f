// Entry points whose kernels are not built yet: they report DTK_ERR_UNSUPPORTED.
#include "dtk_common.cuh"

extern "C" {
dtk_status dtk_mls_batch_create( int32_t, const dtk_mls_options *, const int64_t *, const double *,
                                 const int64_t *, const double *, dtk_stream_t, dtk_mls_batch_handle * )
{
    dtk::set_error( "batch not built yet" );
    return DTK_ERR_UNSUPPORTED;
}
dtk_status dtk_mls_batch_apply( dtk_mls_batch_handle, const double *, double *, int32_t, dtk_stream_t )
{
    return DTK_ERR_UNSUPPORTED;
}
dtk_status dtk_mls_batch_get_csr( dtk_mls_batch_handle, const int32_t **, const int32_t **,
                                  const void **, int64_t *, int32_t * )
{
    return DTK_ERR_UNSUPPORTED;
}
dtk_status dtk_mls_batch_destroy( dtk_mls_batch_handle ) { return DTK_ERR_UNSUPPORTED; }
}
