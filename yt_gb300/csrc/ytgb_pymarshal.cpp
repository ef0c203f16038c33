// ytgb_pymarshal.cpp -- CPython extension _ytgb_marshal: one native pass over
// the bricks a drop-in sampler collected.
//
// yt hands its sampler one PartitionedGrid per call (render_source.py:594-596)
// and the sampler reads the grid's float64 arrays in place
// (partitioned_grid.pyx:28-63).  The device path needs, for every brick, the
// address and length of each field, the mask, the edges and the dims; a
// Python loop over ~1000 bricks spends a couple of milliseconds on attribute
// and type checks alone.  scan() does the same checks through the buffer
// protocol in C, on (data, mask, left_edge, right_edge, dims) tuples or on
// the PartitionedGrid objects themselves, and writes flat arrays the caller
// allocated.  A brick that
// is not in the expected form (a field that is not a C-contiguous native
// float64 buffer, a mask that is not C-contiguous uint8, edges or dims that
// are not 3 numbers, more than 6 fields) makes scan() return False, and the
// caller takes its Python path for the whole list, which converts such
// arrays.  No reference is kept: the caller keeps the bricks alive.
#define PY_SSIZE_T_CLEAN
#include <Python.h>

#include <cstdint>
#include <cstring>

namespace {

// address and element count of a C-contiguous buffer of item format fmt
// (one char code, optionally with a native byte-order prefix)
bool c_buffer(PyObject *o, char fmt, Py_ssize_t itemsize, uintptr_t *ptr, int64_t *count) {
    Py_buffer v;
    if (PyObject_GetBuffer(o, &v, PyBUF_C_CONTIGUOUS | PyBUF_FORMAT) != 0) {
        PyErr_Clear();
        return false;
    }
    const char *f = v.format ? v.format : "B";
    if (f[0] == '@' || f[0] == '=' || f[0] == '<') f++;  // little-endian hosts only build this
    const bool ok = f[0] == fmt && f[1] == '\0' && v.itemsize == itemsize;
    if (ok) {
        *ptr = (uintptr_t)v.buf;
        *count = (int64_t)(v.len / itemsize);
    }
    PyBuffer_Release(&v);
    return ok;
}

bool three_doubles(PyObject *o, double out[3]) {
    uintptr_t p;
    int64_t n;
    if (c_buffer(o, 'd', 8, &p, &n)) {
        if (n < 3) return false;
        std::memcpy(out, (const void *)p, 3 * sizeof(double));
        return true;
    }
    PyObject *seq = PySequence_Fast(o, "edges");
    if (!seq) {
        PyErr_Clear();
        return false;
    }
    bool ok = PySequence_Fast_GET_SIZE(seq) >= 3;
    for (int i = 0; ok && i < 3; i++) {
        out[i] = PyFloat_AsDouble(PySequence_Fast_GET_ITEM(seq, i));
        if (out[i] == -1.0 && PyErr_Occurred()) {
            PyErr_Clear();
            ok = false;
        }
    }
    Py_DECREF(seq);
    return ok;
}

bool three_ints(PyObject *o, int64_t out[3]) {
    PyObject *seq = PySequence_Fast(o, "dims");
    if (!seq) {
        PyErr_Clear();
        return false;
    }
    bool ok = PySequence_Fast_GET_SIZE(seq) == 3;
    for (int i = 0; ok && i < 3; i++) {
        out[i] = PyLong_AsLongLong(PySequence_Fast_GET_ITEM(seq, i));
        if (out[i] == -1 && PyErr_Occurred()) {
            PyErr_Clear();
            ok = false;
        }
    }
    Py_DECREF(seq);
    return ok;
}

// One brick as (data, mask, left_edge, right_edge, dims): a 5-tuple, or an
// object with yt's PartitionedGrid attributes my_data, source_mask,
// LeftEdge and RightEdge (dims from the mask's shape).  New references in
// out[0..4]; false when the object is neither.
bool brick_parts(PyObject *t, PyObject *out[5]) {
    if (PyTuple_Check(t)) {
        if (PyTuple_GET_SIZE(t) != 5) return false;
        for (int i = 0; i < 5; i++) {
            out[i] = PyTuple_GET_ITEM(t, i);
            Py_INCREF(out[i]);
        }
        return true;
    }
    static PyObject *names[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    if (!names[0]) {
        const char *s[5] = {"my_data", "source_mask", "LeftEdge", "RightEdge", "shape"};
        for (int i = 0; i < 5; i++) names[i] = PyUnicode_InternFromString(s[i]);
    }
    for (int i = 0; i < 4; i++) {
        out[i] = PyObject_GetAttr(t, names[i]);
        if (!out[i]) {
            PyErr_Clear();
            for (int j = 0; j < i; j++) Py_DECREF(out[j]);
            return false;
        }
    }
    out[4] = PyObject_GetAttr(out[1], names[4]);
    if (!out[4]) {
        PyErr_Clear();
        for (int j = 0; j < 4; j++) Py_DECREF(out[j]);
        return false;
    }
    return true;
}

// scan(bricks, field_cap, fptr, fsize, nfields, dims, le, re, mptr, msize)
// bricks: sequence of (data, mask, left_edge, right_edge, dims) tuples or
// PartitionedGrid-like objects.
// The others are addresses of caller arrays: fptr (uint64) / fsize (int64)
// of field_cap entries; nfields (int64), mptr (uint64), msize (int64; -1 for
// no mask) of len(bricks) entries; dims (int64), le, re (float64) of
// 3 len(bricks).  Returns the number of fields, or False.
PyObject *scan(PyObject *, PyObject *args) {
    PyObject *bricks;
    Py_ssize_t cap;
    unsigned long long a_fptr, a_fsize, a_nf, a_dims, a_le, a_re, a_mptr, a_msz;
    if (!PyArg_ParseTuple(args, "OnKKKKKKKK", &bricks, &cap, &a_fptr, &a_fsize, &a_nf, &a_dims, &a_le, &a_re,
                          &a_mptr, &a_msz))
        return nullptr;
    PyObject *seq = PySequence_Fast(bricks, "bricks must be a sequence");
    if (!seq) return nullptr;
    uint64_t *fptr = (uint64_t *)(uintptr_t)a_fptr;
    int64_t *fsize = (int64_t *)(uintptr_t)a_fsize;
    int64_t *nf = (int64_t *)(uintptr_t)a_nf;
    int64_t *dims = (int64_t *)(uintptr_t)a_dims;
    double *le = (double *)(uintptr_t)a_le;
    double *re = (double *)(uintptr_t)a_re;
    uint64_t *mptr = (uint64_t *)(uintptr_t)a_mptr;
    int64_t *msz = (int64_t *)(uintptr_t)a_msz;
    const Py_ssize_t n = PySequence_Fast_GET_SIZE(seq);
    Py_ssize_t nfield = 0;
    bool ok = true;
    for (Py_ssize_t k = 0; ok && k < n; k++) {
        PyObject *part[5];
        if (!brick_parts(PySequence_Fast_GET_ITEM(seq, k), part)) {
            ok = false;
            break;
        }
        PyObject *data = PySequence_Fast(part[0], "fields");
        if (!data) {
            PyErr_Clear();
            for (int i = 0; i < 5; i++) Py_DECREF(part[i]);
            ok = false;
            break;
        }
        const Py_ssize_t m = PySequence_Fast_GET_SIZE(data);
        ok = m >= 1 && m <= 6 && nfield + m <= cap;
        for (Py_ssize_t f = 0; ok && f < m; f++) {
            uintptr_t p;
            int64_t c;
            ok = c_buffer(PySequence_Fast_GET_ITEM(data, f), 'd', 8, &p, &c);
            if (ok) {
                fptr[nfield] = p;
                fsize[nfield] = c;
                nfield++;
            }
        }
        Py_DECREF(data);
        if (!ok) {
            for (int i = 0; i < 5; i++) Py_DECREF(part[i]);
            break;
        }
        nf[k] = m;
        PyObject *mask = part[1];
        if (mask == Py_None) {
            mptr[k] = 0;
            msz[k] = -1;
        } else {
            uintptr_t p;
            int64_t c;
            ok = c_buffer(mask, 'B', 1, &p, &c);
            mptr[k] = p;
            msz[k] = c;
        }
        ok = ok && three_doubles(part[2], le + 3 * k) && three_doubles(part[3], re + 3 * k) &&
             three_ints(part[4], dims + 3 * k);
        for (int i = 0; i < 5; i++) Py_DECREF(part[i]);
    }
    Py_DECREF(seq);
    if (!ok) Py_RETURN_FALSE;
    return PyLong_FromSsize_t(nfield);
}

PyMethodDef methods[] = {
    {"scan", scan, METH_VARARGS, "Flatten (data, mask, left_edge, right_edge, dims) bricks into caller arrays."},
    {nullptr, nullptr, 0, nullptr},
};

PyModuleDef module = {PyModuleDef_HEAD_INIT, "_ytgb_marshal", "Native brick marshalling for yt_gb300.", -1, methods};

}  // namespace

PyMODINIT_FUNC PyInit__ytgb_marshal(void) { return PyModule_Create(&module); }
