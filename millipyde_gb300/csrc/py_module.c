/*
 * py_module.c -- module init and module-level functions
 * (reference src/millipyde_module.c:112-301).
 *
 * Unlike the reference, importing succeeds on a machine without a GPU:
 * DEVICE_COUNT is then 0 and every call that needs the device raises
 * RuntimeError("no CUDA device is available").
 */
#define MP_MAIN_MODULE
#include "py_common.h"

static PyObject *mpmod_device_count(PyObject *self, PyObject *unused)
{
    return PyLong_FromLong(mpdev_get_device_count());
}

static PyObject *mpmod_get_current_device(PyObject *self, PyObject *unused)
{
    int d = mpdev_get_target_device();
    if (d == DEVICE_LOC_NO_AFFINITY) d = mpdev_get_recommended_device();
    return PyLong_FromLong(d);
}

static PyObject *mpmod_best_device(PyObject *self, PyObject *unused)
{
    return PyLong_FromLong(mpdev_get_recommended_device());
}

static PyObject *mpmod_seed(PyObject *self, PyObject *arg)
{
    unsigned long long v = PyLong_AsUnsignedLongLongMask(arg);
    if (PyErr_Occurred()) return NULL;
    mp_seed((uint64_t)v);
    Py_RETURN_NONE;
}

static PyObject *mpmod_synchronize(PyObject *self, PyObject *unused)
{
    MPStatus st;
    Py_BEGIN_ALLOW_THREADS
    st = mpdev_synchronize();
    Py_END_ALLOW_THREADS
    if (st != MILLIPYDE_SUCCESS) return mp_raise(st);
    Py_RETURN_NONE;
}

/* _counter_uniform(seed, index, stage, slot): the batch RNG, for tests. */
static PyObject *mpmod_counter_uniform(PyObject *self, PyObject *args)
{
    unsigned long long seed, index;
    unsigned int stage, slot;
    if (!PyArg_ParseTuple(args, "KKII", &seed, &index, &stage, &slot)) return NULL;
    return PyFloat_FromDouble(mp_counter_uniform(seed, index, stage, slot));
}

/*
 * _png_unfilter(data, height, stride, bpp) -> bytes: reverses the PNG row
 * filters (None, Sub, Up, Average, Paeth; PNG specification, section 9)
 * of a decompressed IDAT stream of `height` rows, each a filter byte then
 * `stride` bytes, `bpp` bytes per complete pixel.  The image loader's only
 * per-pixel loop, in C (the reference decoded files with scikit-image).
 */
static PyObject *mpmod_png_unfilter(PyObject *self, PyObject *args)
{
    Py_buffer in;
    Py_ssize_t h, stride, bpp;
    if (!PyArg_ParseTuple(args, "y*nnn", &in, &h, &stride, &bpp)) return NULL;
    if (h < 0 || stride < 0 || bpp < 1 || bpp > 8 || in.len < h * (stride + 1)) {
        PyBuffer_Release(&in);
        PyErr_SetString(PyExc_ValueError, "PNG data shorter than its header says");
        return NULL;
    }
    PyObject *out = PyBytes_FromStringAndSize(NULL, h * stride);
    if (!out) {
        PyBuffer_Release(&in);
        return NULL;
    }
    const unsigned char *src = (const unsigned char *)in.buf;
    unsigned char *dst = (unsigned char *)PyBytes_AS_STRING(out);
    int bad = 0;
    Py_BEGIN_ALLOW_THREADS
    for (Py_ssize_t y = 0; y < h && !bad; ++y) {
        const unsigned char ft = src[y * (stride + 1)];
        const unsigned char *line = src + y * (stride + 1) + 1;
        unsigned char *cur = dst + y * stride;
        const unsigned char *prev = y ? dst + (y - 1) * stride : NULL;
        for (Py_ssize_t x = 0; x < stride; ++x) {
            const int a = x >= bpp ? cur[x - bpp] : 0;
            const int b = prev ? prev[x] : 0;
            const int c = (prev && x >= bpp) ? prev[x - bpp] : 0;
            int v;
            switch (ft) {
            case 0: v = 0; break;
            case 1: v = a; break;
            case 2: v = b; break;
            case 3: v = (a + b) >> 1; break;
            case 4: {
                const int p = a + b - c;
                const int pa = abs(p - a), pb = abs(p - b), pc = abs(p - c);
                v = (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
                break;
            }
            default: v = 0; bad = 1; break;
            }
            cur[x] = (unsigned char)(line[x] + v);
        }
    }
    Py_END_ALLOW_THREADS
    PyBuffer_Release(&in);
    if (bad) {
        Py_DECREF(out);
        PyErr_SetString(PyExc_ValueError, "unknown PNG row filter");
        return NULL;
    }
    return out;
}

static PyMethodDef MillipydeMethods[] = {
    {"_png_unfilter", mpmod_png_unfilter, METH_VARARGS, "Reverse the PNG row filters (image loading)."},
    {"device_count", mpmod_device_count, METH_NOARGS, "Number of usable GPUs."},
    {"get_current_device", mpmod_get_current_device, METH_NOARGS, "Target device id."},
    {"best_device", mpmod_best_device, METH_NOARGS, "Recommended device id."},
    {"seed", mpmod_seed, METH_O, "Seed the random_* methods and probabilistic Operations."},
    {"synchronize", mpmod_synchronize, METH_NOARGS, "Wait for all queued GPU work."},
    {"_counter_uniform", mpmod_counter_uniform, METH_VARARGS, "Counter RNG draw (testing)."},
    {NULL, NULL, 0, NULL}};

static struct PyModuleDef millipydeModule = {
    PyModuleDef_HEAD_INIT, "_millipyde",
    "GB300-native implementation of millipyde's GPU image types.", -1, MillipydeMethods};

PyMODINIT_FUNC PyInit__millipyde(void)
{
    import_array();
    mpdev_initialize();   /* no GPU is not an import error */

    if (PyType_Ready(&PyGPUArray_Type) < 0) return NULL;
    PyGPUImage_Type.tp_base = &PyGPUArray_Type;
    if (PyType_Ready(&PyGPUImage_Type) < 0) return NULL;
    if (PyType_Ready(&PyGPUOperation_Type) < 0) return NULL;
    if (PyType_Ready(&PyGPUPipeline_Type) < 0) return NULL;
    if (PyType_Ready(&PyGPUGenerator_Type) < 0) return NULL;
    if (PyType_Ready(&PyDevice_Type) < 0) return NULL;

    PyObject *m = PyModule_Create(&millipydeModule);
    if (!m) return NULL;
    PyModule_AddIntConstant(m, "DEVICE_COUNT", (long)mpdev_get_device_count());

    struct { const char *name; PyTypeObject *type; } types[] = {
        {"gpuarray", &PyGPUArray_Type},   {"gpuimage", &PyGPUImage_Type},
        {"Operation", &PyGPUOperation_Type}, {"Pipeline", &PyGPUPipeline_Type},
        {"Generator", &PyGPUGenerator_Type}, {"Device", &PyDevice_Type},
    };
    for (size_t i = 0; i < sizeof(types) / sizeof(types[0]); ++i) {
        Py_INCREF(types[i].type);
        if (PyModule_AddObject(m, types[i].name, (PyObject *)types[i].type) < 0) {
            Py_DECREF(types[i].type);
            Py_DECREF(m);
            return NULL;
        }
    }
    return m;
}
