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

static PyMethodDef MillipydeMethods[] = {
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
