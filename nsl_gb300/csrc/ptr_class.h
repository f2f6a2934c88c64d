/* Classification of a caller buffer for the handle's GPU, from the fields cudaPointerGetAttributes reports.
 * Plain C with no CUDA types, so that host-only tests can check the rule without a GPU. */
#ifndef NSLG_PTR_CLASS_H
#define NSLG_PTR_CLASS_H

enum { NSLG_PTR_HOST = 0, NSLG_PTR_DEVICE = 1, NSLG_PTR_FOREIGN = 2 };

/* is_device_memory: the attributes say cudaMemoryTypeDevice; is_managed: cudaMemoryTypeManaged; ptr_device: the
 * attributes' device ordinal; ctx_device: the ordinal the handle runs on. Managed memory is addressable from every
 * GPU; device memory only from its own GPU (the library enables no peer access); anything else is host memory,
 * which the entry points stage through the handle's workspace. */
static inline int nslg_ptr_class(int is_device_memory, int is_managed, int ptr_device, int ctx_device) {
    if (is_managed) return NSLG_PTR_DEVICE;
    if (!is_device_memory) return NSLG_PTR_HOST;
    return ptr_device == ctx_device ? NSLG_PTR_DEVICE : NSLG_PTR_FOREIGN;
}

#endif
