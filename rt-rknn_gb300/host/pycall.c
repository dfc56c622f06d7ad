// CPython entry point for rknn_query_batch with buffer-protocol inputs (numpy
// arrays of int32 query ids and k values).  The ctypes route costs several
// microseconds a call in Python (a pointer object per array, conversion of
// nine arguments), a large share of the host time of a 1000-query call; this
// one parses the arguments in C and releases the interpreter lock around the
// query.  rknn.py uses it when it was built (the CPython headers are needed)
// and ctypes otherwise: both call the same C entry point.
#define PY_SSIZE_T_CLEAN
#include <Python.h>
#include <stdint.h>

#include "rknn_gpu.h"

// query_batch(index, q, k, mode, out_ids, cap, offsets) -> status
//   index, out_ids, offsets: addresses (int); q, k: C-contiguous int32
//   buffers of equal length; cap: the capacity of out_ids in ids.
static PyObject* query_batch(PyObject* self, PyObject* args)
{
    (void)self;
    unsigned long long h = 0, out = 0, off = 0;
    long long cap = 0;
    int mode = 0;
    Py_buffer qb, kb;
    if (!PyArg_ParseTuple(args, "Ky*y*iKLK", &h, &qb, &kb, &mode, &out, &cap, &off)) return NULL;
    rknn_status rc = RKNN_ERR_ARG;
    if (qb.len % 4 == 0 && kb.len == qb.len && qb.len / 4 <= INT32_MAX) {
        Py_BEGIN_ALLOW_THREADS
        rc = rknn_query_batch((rknn_index*)(uintptr_t)h, (const int32_t*)qb.buf, (const int32_t*)kb.buf,
                              (int32_t)(qb.len / 4), (int32_t)mode, (int32_t*)(uintptr_t)out, (int64_t)cap,
                              (int64_t*)(uintptr_t)off, NULL);
        Py_END_ALLOW_THREADS
    }
    PyBuffer_Release(&qb);
    PyBuffer_Release(&kb);
    return PyLong_FromLong((long)rc);
}

static PyMethodDef methods[] = {
    {"query_batch", query_batch, METH_VARARGS, "rknn_query_batch on int32 buffers; returns the status"},
    {NULL, NULL, 0, NULL},
};

static struct PyModuleDef module = {PyModuleDef_HEAD_INIT, "_rknn_call", NULL, -1, methods, NULL, NULL, NULL, NULL};

PyMODINIT_FUNC PyInit__rknn_call(void) { return PyModule_Create(&module); }
