/*
 * py_compose.c -- Operation, Pipeline, Generator and Device.
 *
 * Operation (src/gpuoperation.c): a deferred call with a probability.
 * Pipeline  (src/gpupipeline.c):  applies a list of Operations to a list of
 *           images.  run() lowers the string-named image ops to MPStage
 *           records and hands the whole batch to the fused C-ABI path
 *           (mpk_pipeline_run_objects) instead of one host thread and one
 *           stream sync per image and stage.  random_* names run too (the
 *           reference silently skipped them, src/gpupipeline.c:375).
 * Generator (src/gpugenerator.c): produces clones of inputs[i % n] with the
 *           operations applied.  When every operation is an image op and the
 *           inputs are float32 images it produces a batch of outputs with one
 *           fused run; output i draws its random parameters from (seed, i), so
 *           results do not depend on the batch size.
 * Device    (src/device.c): `with Device(i):` sets the target device.
 */
#include "py_common.h"

#include <string.h>

/* ======================================================================== */
/* Operation                                                                */
/* ======================================================================== */
static void PyGPUOperation_dealloc(PyGPUOperationObject *self)
{
    Py_XDECREF(self->callable);
    Py_XDECREF(self->arg_tuple);
    Py_TYPE(self)->tp_free((PyObject *)self);
}

static PyObject *PyGPUOperation_new(PyTypeObject *type, PyObject *args, PyObject *kwds)
{
    PyGPUOperationObject *self = (PyGPUOperationObject *)type->tp_alloc(type, 0);
    if (self) {
        self->callable = NULL;
        self->arg_tuple = NULL;
        self->requires_instance = MP_FALSE;
        self->probability = -1.0;
    }
    return (PyObject *)self;
}

/* Operation(callable_or_name, *args, probability=p); p a float in (0, 1)
 * (src/gpuoperation.c:44-122). */
static int PyGPUOperation_init(PyGPUOperationObject *self, PyObject *args, PyObject *kwds)
{
    Py_ssize_t n = PyTuple_Size(args);
    if (n < 1) {
        PyErr_SetString(PyExc_ValueError, mperr_str(GPUOPERATION_ERROR_CONSTRUCTION_NO_ARGS));
        return -1;
    }
    double prob = -1.0;
    if (kwds && PyDict_Size(kwds) > 0) {
        PyObject *p = PyDict_GetItemString(kwds, "probability");
        if (!p || PyDict_Size(kwds) != 1) {
            PyErr_SetString(PyExc_ValueError, mperr_str(GPUOPERATION_ERROR_CONSTRUCTION_NAMED_ARGS));
            return -1;
        }
        if (!PyFloat_Check(p)) {
            PyErr_SetString(PyExc_ValueError, mperr_str(GPUOPERATION_ERROR_INVALID_PROBABILITY));
            return -1;
        }
        prob = PyFloat_AsDouble(p);
        if (!(prob > 0.0 && prob < 1.0)) {
            PyErr_SetString(PyExc_ValueError, mperr_str(GPUOPERATION_ERROR_INVALID_PROBABILITY));
            return -1;
        }
    }
    PyObject *callable = PyTuple_GET_ITEM(args, 0);
    PyObject *rest = PyTuple_GetSlice(args, 1, n);
    if (!rest) return -1;
    Py_INCREF(callable);
    Py_XSETREF(self->callable, callable);
    Py_XSETREF(self->arg_tuple, rest);
    self->requires_instance = PyUnicode_Check(callable) ? MP_TRUE : MP_FALSE;
    self->probability = prob;
    return 0;
}

MPStatus gpuoperation_evaluate_probability(MPBool *result, double probability)
{
    *result = MP_TRUE;
    if (probability < 0) return MILLIPYDE_SUCCESS;
    double r;
    MPStatus st = random_double_in_range(0.0, 1.0, &r);
    if (st != MILLIPYDE_SUCCESS) return st;
    if (r > probability) *result = MP_FALSE;
    return MILLIPYDE_SUCCESS;
}

static PyObject *mp_operation_call(PyGPUOperationObject *self, PyObject *callable)
{
    MPBool run;
    MPStatus st = gpuoperation_evaluate_probability(&run, self->probability);
    if (st != MILLIPYDE_SUCCESS) {
        PyErr_SetString(PyExc_RuntimeError, mperr_str(st));
        return NULL;
    }
    if (!run) Py_RETURN_NONE;
    return PyObject_Call(callable, self->arg_tuple, NULL);
}

PyObject *PyGPUOperation_run(PyGPUOperationObject *self, PyObject *unused)
{
    return mp_operation_call(self, self->callable);
}

PyObject *PyGPUOperation_run_on(PyGPUOperationObject *self, PyObject *instance)
{
    if (!PyUnicode_Check(self->callable)) {
        PyErr_SetString(PyExc_ValueError, mperr_str(GPUOPERATION_ERROR_RUN_WITHOUT_STRING_METHOD));
        return NULL;
    }
    PyObject *m = PyObject_GetAttr(instance, self->callable);
    if (!m) {
        PyErr_Clear();
        PyErr_SetString(PyExc_ValueError, mperr_str(GPUOPERATION_ERROR_RUN_UNKNOWN_STRING_METHOD));
        return NULL;
    }
    PyObject *r = mp_operation_call(self, m);
    Py_DECREF(m);
    return r;
}

static int mp_args_d(PyObject *t, int need, double *out)
{
    if (PyTuple_Size(t) != need) return -1;
    for (int i = 0; i < need; ++i) {
        out[i] = PyFloat_AsDouble(PyTuple_GET_ITEM(t, i));
        if (PyErr_Occurred()) return -1;
    }
    return 0;
}

static int mp_pair(PyObject *o, double *lo, double *hi)
{
    PyObject *seq = PySequence_Fast(o, "expected a [min, max] list");
    if (!seq) return -1;
    int ok = PySequence_Fast_GET_SIZE(seq) == 2;
    if (ok) {
        *lo = PyFloat_AsDouble(PySequence_Fast_GET_ITEM(seq, 0));
        *hi = PyFloat_AsDouble(PySequence_Fast_GET_ITEM(seq, 1));
    }
    Py_DECREF(seq);
    if (!ok || PyErr_Occurred()) return -1;
    return 0;
}

/* Name + arguments -> MPStage (the reference's name tables,
 * src/gpuoperation.c:213-291, plus the random_* names). */
int mp_stage_from_operation(PyGPUOperationObject *op, MPStage *s)
{
    if (!op->requires_instance) return 0;
    const char *name = PyUnicode_AsUTF8(op->callable);
    if (!name) return -1;
    PyObject *a = op->arg_tuple;
    memset(s, 0, sizeof(*s));
    s->probability = op->probability;
    double v[3];
#define MP_BAD_ARGS                                                                    \
    do {                                                                               \
        if (!PyErr_Occurred())                                                         \
            PyErr_Format(PyExc_TypeError, "bad arguments for operation '%s'", name);   \
        return -1;                                                                     \
    } while (0)
    if (!strcmp(name, "rgb2grey") || !strcmp(name, "rgb2gray") || !strcmp(name, "rgba2grey") ||
        !strcmp(name, "rgba2gray")) {
        s->op = MP_OP_RGB2GREY;
    } else if (!strcmp(name, "transpose")) {
        s->op = MP_OP_TRANSPOSE;
    } else if (!strcmp(name, "fliplr")) {
        s->op = MP_OP_FLIPLR;
    } else if (!strcmp(name, "gaussian")) {
        if (mp_args_d(a, 1, v) < 0) MP_BAD_ARGS;
        if (!(v[0] > 0)) { PyErr_SetString(PyExc_ValueError, "gaussian sigma must be positive"); return -1; }
        s->op = MP_OP_GAUSSIAN; s->lo[0] = v[0];
    } else if (!strcmp(name, "rotate")) {
        if (mp_args_d(a, 1, v) < 0) MP_BAD_ARGS;
        s->op = MP_OP_ROTATE; s->lo[0] = v[0];
    } else if (!strcmp(name, "brightness")) {
        if (mp_args_d(a, 1, v) < 0) MP_BAD_ARGS;
        if (v[0] <= -1.0 || v[0] >= 1.0) {
            PyErr_SetString(PyExc_ValueError, "brightness delta must lie strictly between -1 and 1");
            return -1;
        }
        s->op = MP_OP_BRIGHTNESS; s->lo[0] = v[0];
    } else if (!strcmp(name, "adjust_gamma")) {
        if (PyTuple_Size(a) == 1) { if (mp_args_d(a, 1, v) < 0) MP_BAD_ARGS; v[1] = 1.0; }
        else if (mp_args_d(a, 2, v) < 0) MP_BAD_ARGS;
        s->op = MP_OP_ADJUST_GAMMA; s->lo[0] = v[0]; s->lo[1] = v[1];
    } else if (!strcmp(name, "colorize")) {
        if (mp_args_d(a, 3, v) < 0) MP_BAD_ARGS;
        if (v[0] < 0 || v[1] < 0 || v[2] < 0) {
            PyErr_SetString(PyExc_ValueError, "colorize multipliers must be non-negative");
            return -1;
        }
        s->op = MP_OP_COLORIZE; s->lo[0] = v[0]; s->lo[1] = v[1]; s->lo[2] = v[2];
    } else if (!strcmp(name, "random_rotate") || !strcmp(name, "random_gaussian") ||
               !strcmp(name, "random_brightness")) {
        if (mp_args_d(a, 2, v) < 0) MP_BAD_ARGS;
        s->op = !strcmp(name, "random_rotate") ? MP_OP_ROTATE
              : !strcmp(name, "random_gaussian") ? MP_OP_GAUSSIAN : MP_OP_BRIGHTNESS;
        s->random = 1;
        s->lo[0] = v[0]; s->hi[0] = v[1];
        if (s->op == MP_OP_GAUSSIAN && !(v[0] > 0 && v[1] > 0)) {
            PyErr_SetString(PyExc_ValueError, "gaussian sigma range must be positive");
            return -1;
        }
    } else if (!strcmp(name, "random_adjust_gamma")) {
        if (PyTuple_Size(a) != 2) MP_BAD_ARGS;
        PyObject *a0 = PyTuple_GET_ITEM(a, 0), *a1 = PyTuple_GET_ITEM(a, 1);
        s->op = MP_OP_ADJUST_GAMMA; s->random = 1;
        if (PySequence_Check(a0) && PySequence_Check(a1)) {
            if (mp_pair(a0, &s->lo[0], &s->hi[0]) < 0 || mp_pair(a1, &s->lo[1], &s->hi[1]) < 0) MP_BAD_ARGS;
        } else {
            if (mp_args_d(a, 2, v) < 0) MP_BAD_ARGS;
            s->lo[0] = v[0]; s->hi[0] = v[1]; s->lo[1] = s->hi[1] = 1.0;
        }
    } else if (!strcmp(name, "random_colorize")) {
        if (PyTuple_Size(a) != 3) MP_BAD_ARGS;
        s->op = MP_OP_COLORIZE; s->random = 1;
        for (int k = 0; k < 3; ++k)
            if (mp_pair(PyTuple_GET_ITEM(a, k), &s->lo[k], &s->hi[k]) < 0) MP_BAD_ARGS;
    } else {
        return 0;
    }
#undef MP_BAD_ARGS
    return 1;
}

static PyMethodDef PyGPUOperation_methods[] = {
    {"run", (PyCFunction)PyGPUOperation_run, METH_NOARGS, "Call the stored callable with its arguments."},
    {"run_on", (PyCFunction)PyGPUOperation_run_on, METH_O,
     "Call the named method on the given object with the stored arguments."},
    {NULL}};

static PyMemberDef PyGPUOperation_members[] = {
    {"probability", T_DOUBLE, offsetof(PyGPUOperationObject, probability), READONLY,
     "probability of running (-1: always)"},
    {NULL}};

PyTypeObject PyGPUOperation_Type = {
    PyVarObject_HEAD_INIT(NULL, 0).tp_name = "millipyde.Operation",
    .tp_basicsize = sizeof(PyGPUOperationObject),
    .tp_dealloc = (destructor)PyGPUOperation_dealloc,
    .tp_flags = Py_TPFLAGS_DEFAULT,
    .tp_doc = "Operation(method_name_or_callable, *args, probability=p)",
    .tp_methods = PyGPUOperation_methods,
    .tp_members = PyGPUOperation_members,
    .tp_init = (initproc)PyGPUOperation_init,
    .tp_new = PyGPUOperation_new,
};

/* ======================================================================== */
/* Pipeline                                                                 */
/* ======================================================================== */
static void PyGPUPipeline_dealloc(PyGPUPipelineObject *self)
{
    Py_XDECREF(self->inputs);
    Py_XDECREF(self->operations);
    Py_XDECREF((PyObject *)self->receiver);
    Py_TYPE(self)->tp_free((PyObject *)self);
}

static PyObject *PyGPUPipeline_new(PyTypeObject *type, PyObject *args, PyObject *kwds)
{
    PyGPUPipelineObject *self = (PyGPUPipelineObject *)type->tp_alloc(type, 0);
    if (self) {
        self->device_id = DEVICE_LOC_NO_AFFINITY;
        self->receiver = NULL;
        self->has_seed = 0;
        self->seed = 0;
        self->runs = 0;
    }
    return (PyObject *)self;
}

static int mp_parse_device(PyObject *d, MPStatus bad_type, MPStatus unusable, int *out)
{
    if (!PyLong_Check(d) || PyBool_Check(d)) {
        PyErr_SetString(PyExc_ValueError, mperr_str(bad_type));
        return -1;
    }
    long v = PyLong_AsLong(d);
    if (PyErr_Occurred() || !mpdev_is_valid_device((int)v)) {
        PyErr_Clear();
        PyErr_SetString(PyExc_ValueError, mperr_str(unusable));
        return -1;
    }
    *out = (int)v;
    return 0;
}

static int mp_parse_seed(PyObject *s, uint64_t *out)
{
    unsigned long long v = PyLong_AsUnsignedLongLongMask(s);
    if (PyErr_Occurred()) return -1;
    *out = (uint64_t)v;
    return 0;
}

/* Pipeline(inputs, operations, device=None, seed=None)
 * (src/gpupipeline.c:56-167). */
static int PyGPUPipeline_init(PyGPUPipelineObject *self, PyObject *args, PyObject *kwds)
{
    Py_ssize_t n = PyTuple_Size(args);
    if (n < 2 || n > 3) {
        PyErr_SetString(PyExc_ValueError, mperr_str(GPUPIPELINE_ERROR_CONSTRUCTION_INVALID_ARGS));
        return -1;
    }
    PyObject *inputs = PyTuple_GET_ITEM(args, 0);
    PyObject *ops = PyTuple_GET_ITEM(args, 1);
    if (!PyList_CheckExact(inputs)) {
        PyErr_SetString(PyExc_ValueError, mperr_str(GPUPIPELINE_ERROR_NONLIST_INPUTS));
        return -1;
    }
    if (!PyList_CheckExact(ops)) {
        PyErr_SetString(PyExc_ValueError, mperr_str(GPUPIPELINE_ERROR_NONLIST_OPERATIONS));
        return -1;
    }
    self->device_id = mpdev_get_target_device();
    if (n == 3 && mp_parse_device(PyTuple_GET_ITEM(args, 2), GPUPIPELINE_ERROR_INVALID_DEVICE,
                                  GPUPIPELINE_ERROR_UNUSABLE_DEVICE, &self->device_id) < 0)
        return -1;
    if (kwds && PyDict_Size(kwds) > 0) {
        PyObject *k, *v;
        Py_ssize_t pos = 0;
        while (PyDict_Next(kwds, &pos, &k, &v)) {
            const char *key = PyUnicode_AsUTF8(k);
            if (key && !strcmp(key, "device")) {
                if (mp_parse_device(v, GPUPIPELINE_ERROR_INVALID_DEVICE,
                                    GPUPIPELINE_ERROR_UNUSABLE_DEVICE, &self->device_id) < 0)
                    return -1;
            } else if (key && !strcmp(key, "seed")) {
                if (v != Py_None) {
                    if (mp_parse_seed(v, &self->seed) < 0) return -1;
                    self->has_seed = 1;
                }
            } else {
                PyErr_SetString(PyExc_ValueError, mperr_str(GPUPIPELINE_ERROR_CONSTRUCTION_NAMED_ARGS));
                return -1;
            }
        }
    }
    for (Py_ssize_t i = 0; i < PyList_GET_SIZE(inputs); ++i) {
        if (!mp_is_gpuarray(PyList_GET_ITEM(inputs, i))) {
            PyErr_SetString(PyExc_ValueError, mperr_str(GPUPIPELINE_ERROR_NONGPU_INPUT));
            return -1;
        }
    }
    for (Py_ssize_t i = 0; i < PyList_GET_SIZE(ops); ++i) {
        if (!PyObject_TypeCheck(PyList_GET_ITEM(ops, i), &PyGPUOperation_Type)) {
            PyErr_SetString(PyExc_ValueError, mperr_str(GPUPIPELINE_ERROR_NONLIST_OPERATIONS));
            return -1;
        }
    }
    Py_INCREF(inputs);
    Py_XSETREF(self->inputs, inputs);
    Py_INCREF(ops);
    Py_XSETREF(self->operations, ops);
    return 0;
}

/* Pipeline.connect_to(other): running self then applies other's operations
 * to self's inputs (src/gpupipeline.c:185-218; one GPU, same device). */
static PyObject *PyGPUPipeline_connect_to(PyGPUPipelineObject *self, PyObject *other)
{
    if (!PyObject_TypeCheck(other, &PyGPUPipeline_Type)) {
        PyErr_SetString(PyExc_TypeError, "connect_to needs a Pipeline");
        return NULL;
    }
    for (PyGPUPipelineObject *p = (PyGPUPipelineObject *)other; p; p = p->receiver)
        if (p == self) {
            PyErr_SetString(PyExc_ValueError, "connect_to would create a cycle");
            return NULL;
        }
    Py_INCREF(other);
    Py_XSETREF(self->receiver, (PyGPUPipelineObject *)other);
    Py_RETURN_NONE;
}

/* Appends the batchable stages of `ops` to *stages. */
static int mp_collect_stages(PyObject *ops, MPStage **stages, int *n, int *cap)
{
    for (Py_ssize_t i = 0; i < PyList_GET_SIZE(ops); ++i) {
        PyGPUOperationObject *op = (PyGPUOperationObject *)PyList_GET_ITEM(ops, i);
        MPStage s;
        int r = mp_stage_from_operation(op, &s);
        if (r < 0) return -1;
        if (r == 0) continue;   /* not an image op: skipped, as in the reference */
        if (*n == *cap) {
            *cap = *cap ? *cap * 2 : 16;
            MPStage *ns = (MPStage *)realloc(*stages, sizeof(MPStage) * (size_t)*cap);
            if (!ns) { PyErr_NoMemory(); return -1; }
            *stages = ns;
        }
        (*stages)[(*n)++] = s;
    }
    return 0;
}

static uint64_t mp_fresh_seed(void)
{
    double a, b;
    random_double_in_range(0.0, 4294967296.0, &a);
    random_double_in_range(0.0, 4294967296.0, &b);
    return ((uint64_t)a << 32) ^ (uint64_t)b;
}

static PyObject *mp_pipeline_run_impl(PyGPUPipelineObject *self, int fused)
{
    MPStage *stages = NULL;
    int nst = 0, cap = 0;
    for (PyGPUPipelineObject *p = self; p; p = p->receiver)
        if (mp_collect_stages(p->operations, &stages, &nst, &cap) < 0) { free(stages); return NULL; }
    Py_ssize_t n = PyList_GET_SIZE(self->inputs);
    MPObjData **objs = (MPObjData **)malloc(sizeof(MPObjData *) * (size_t)(n > 0 ? n : 1));
    if (!objs) { free(stages); return PyErr_NoMemory(); }
    for (Py_ssize_t i = 0; i < n; ++i)
        objs[i] = ((PyGPUArrayObject *)PyList_GET_ITEM(self->inputs, i))->obj_data;
    uint64_t seed = self->has_seed ? self->seed : mp_fresh_seed();
    uint64_t index0 = self->has_seed ? self->runs * (uint64_t)n : 0;
    MPStatus st;
    Py_BEGIN_ALLOW_THREADS
    st = mpk_pipeline_run_objects(stages, nst, objs, (int)n, seed, index0, fused);
    Py_END_ALLOW_THREADS
    free(stages);
    free(objs);
    if (st != MILLIPYDE_SUCCESS) return mp_raise(st);
    self->runs++;
    for (Py_ssize_t i = 0; i < n; ++i) {
        PyObject *o = PyList_GET_ITEM(self->inputs, i);
        if (mp_is_gpuimage(o)) {
            MPObjData *d = ((PyGPUArrayObject *)o)->obj_data;
            ((PyGPUImageObject *)o)->height = d->dims[0];
            ((PyGPUImageObject *)o)->width = d->dims[1];
        }
    }
    Py_RETURN_NONE;
}

/* Pipeline.run() (src/gpupipeline.c:233-312).  Returns when the work is
 * queued on the device stream; reading an image back waits for it. */
static PyObject *PyGPUPipeline_run(PyGPUPipelineObject *self, PyObject *unused)
{
    return mp_pipeline_run_impl(self, 1);
}

/* Same stages, one kernel launch per stage and image (the unfused path). */
static PyObject *PyGPUPipeline_run_unfused(PyGPUPipelineObject *self, PyObject *unused)
{
    return mp_pipeline_run_impl(self, 0);
}

static PyMethodDef PyGPUPipeline_methods[] = {
    {"run", (PyCFunction)PyGPUPipeline_run, METH_NOARGS, "Apply the operations to every input."},
    {"run_unfused", (PyCFunction)PyGPUPipeline_run_unfused, METH_NOARGS,
     "Apply the operations with one kernel per stage and image."},
    {"connect_to", (PyCFunction)PyGPUPipeline_connect_to, METH_O,
     "Chain another pipeline's operations after this one's."},
    {NULL}};

PyTypeObject PyGPUPipeline_Type = {
    PyVarObject_HEAD_INIT(NULL, 0).tp_name = "millipyde.Pipeline",
    .tp_basicsize = sizeof(PyGPUPipelineObject),
    .tp_dealloc = (destructor)PyGPUPipeline_dealloc,
    .tp_flags = Py_TPFLAGS_DEFAULT,
    .tp_doc = "Pipeline(inputs, operations, device=None, seed=None)",
    .tp_methods = PyGPUPipeline_methods,
    .tp_init = (initproc)PyGPUPipeline_init,
    .tp_new = PyGPUPipeline_new,
};

/* ======================================================================== */
/* Generator                                                                */
/* ======================================================================== */
#define MP_GEN_BATCH 64
#define MP_GEN_BATCH_BYTES (512ull << 20)

static void PyGPUGenerator_dealloc(PyGPUGeneratorObject *self)
{
    Py_XDECREF(self->inputs);
    Py_XDECREF(self->operations);
    Py_XDECREF(self->ready);
    Py_TYPE(self)->tp_free((PyObject *)self);
}

static PyObject *PyGPUGenerator_new(PyTypeObject *type, PyObject *args, PyObject *kwds)
{
    PyGPUGeneratorObject *self = (PyGPUGeneratorObject *)type->tp_alloc(type, 0);
    if (self) {
        self->device_id = DEVICE_LOC_NO_AFFINITY;
        self->max = NO_OUTPUT_MAX;
        self->i = 0;
        self->return_to_host = MP_FALSE;
        self->ready = NULL;
        self->seed = 0;
    }
    return (PyObject *)self;
}

/* Generator(inputs_or_path, operations, device=, outputs=, return_to_host=,
 * seed=) (src/gpugenerator.c:44-169). */
static int PyGPUGenerator_init(PyGPUGeneratorObject *self, PyObject *args, PyObject *kwds)
{
    Py_ssize_t n = PyTuple_Size(args);
    if (n != 2) {
        PyErr_SetString(PyExc_ValueError, mperr_str(GPUGENERATOR_ERROR_INVALID_INPUT));
        return -1;
    }
    PyObject *inputs = PyTuple_GET_ITEM(args, 0);
    PyObject *ops = PyTuple_GET_ITEM(args, 1);
    int has_seed = 0;
    if (kwds && PyDict_Size(kwds) > 0) {
        PyObject *k, *v;
        Py_ssize_t pos = 0;
        while (PyDict_Next(kwds, &pos, &k, &v)) {
            const char *key = PyUnicode_AsUTF8(k);
            if (key && !strcmp(key, "device")) {
                if (mp_parse_device(v, GPUGENERATOR_ERROR_INVALID_DEVICE,
                                    GPUGENERATOR_ERROR_UNUSABLE_DEVICE, &self->device_id) < 0)
                    return -1;
            } else if (key && !strcmp(key, "outputs")) {
                if (!PyLong_Check(v) || PyBool_Check(v)) {
                    PyErr_SetString(PyExc_ValueError, mperr_str(GPUGENERATOR_ERROR_INVALID_MAX));
                    return -1;
                }
                self->max = PyLong_AsLong(v);
                if (self->max < 0) {
                    PyErr_SetString(PyExc_ValueError, mperr_str(GPUGENERATOR_ERROR_INVALID_MAX));
                    return -1;
                }
            } else if (key && !strcmp(key, "return_to_host")) {
                if (!PyBool_Check(v)) {
                    PyErr_SetString(PyExc_ValueError, mperr_str(GPUGENERATOR_ERROR_INVALID_RETURN_TO));
                    return -1;
                }
                self->return_to_host = PyObject_IsTrue(v) ? MP_TRUE : MP_FALSE;
            } else if (key && !strcmp(key, "seed")) {
                if (v != Py_None) {
                    if (mp_parse_seed(v, &self->seed) < 0) return -1;
                    has_seed = 1;
                }
            } else {
                PyErr_SetString(PyExc_ValueError, mperr_str(GPUGENERATOR_ERROR_CONSTRUCTION_NAMED_ARGS));
                return -1;
            }
        }
    }
    if (!has_seed) self->seed = mp_fresh_seed();
    if (!PyList_CheckExact(inputs) && !PyUnicode_Check(inputs)) {
        PyErr_SetString(PyExc_ValueError, mperr_str(GPUGENERATOR_ERROR_INVALID_INPUT));
        return -1;
    }
    if (!PyList_CheckExact(ops)) {
        PyErr_SetString(PyExc_ValueError, mperr_str(GPUGENERATOR_ERROR_NONLIST_OPERATIONS));
        return -1;
    }
    for (Py_ssize_t i = 0; i < PyList_GET_SIZE(ops); ++i) {
        if (!PyObject_TypeCheck(PyList_GET_ITEM(ops, i), &PyGPUOperation_Type)) {
            PyErr_SetString(PyExc_ValueError, mperr_str(GPUGENERATOR_ERROR_NONLIST_OPERATIONS));
            return -1;
        }
    }
    PyObject *list;
    if (PyUnicode_Check(inputs)) {
        PyObject *mod = PyImport_ImportModule("millipyde_gb300");
        if (!mod) return -1;
        list = PyObject_CallMethod(mod, "images_from_path", "O", inputs);
        Py_DECREF(mod);
        if (!list) return -1;
        if (!PyList_CheckExact(list)) {
            Py_DECREF(list);
            PyErr_SetString(PyExc_ValueError, mperr_str(GPUGENERATOR_ERROR_INVALID_INPUT));
            return -1;
        }
    } else {
        Py_INCREF(inputs);
        list = inputs;
    }
    for (Py_ssize_t i = 0; i < PyList_GET_SIZE(list); ++i) {
        if (!mp_is_gpuarray(PyList_GET_ITEM(list, i))) {
            Py_DECREF(list);
            PyErr_SetString(PyExc_ValueError, mperr_str(TYPE_ERROR_NON_GPUOBJ));
            return -1;
        }
    }
    Py_XSETREF(self->inputs, list);
    Py_INCREF(ops);
    Py_XSETREF(self->operations, ops);
    Py_XSETREF(self->ready, PyList_New(0));
    return self->ready ? 0 : -1;
}

static PyObject *PyGPUGenerator_iter(PyObject *self)
{
    Py_INCREF(self);
    return self;
}

/* All operations are batchable image ops and every input is a float32 image. */
static int mp_gen_batchable(PyGPUGeneratorObject *g, MPStage **stages, int *nst)
{
    int cap = 0;
    *stages = NULL;
    *nst = 0;
    for (Py_ssize_t i = 0; i < PyList_GET_SIZE(g->operations); ++i) {
        PyGPUOperationObject *op = (PyGPUOperationObject *)PyList_GET_ITEM(g->operations, i);
        MPStage s;
        int r = mp_stage_from_operation(op, &s);
        if (r < 0) { free(*stages); *stages = NULL; return -1; }
        if (r == 0) { free(*stages); *stages = NULL; return 0; }
        if (*nst == cap) {
            cap = cap ? cap * 2 : 16;
            MPStage *ns = (MPStage *)realloc(*stages, sizeof(MPStage) * (size_t)cap);
            if (!ns) { free(*stages); *stages = NULL; PyErr_NoMemory(); return -1; }
            *stages = ns;
        }
        (*stages)[(*nst)++] = s;
    }
    for (Py_ssize_t i = 0; i < PyList_GET_SIZE(g->inputs); ++i) {
        PyObject *o = PyList_GET_ITEM(g->inputs, i);
        MPObjData *d = ((PyGPUArrayObject *)o)->obj_data;
        if (!mp_is_gpuimage(o) || !d || d->type != NPY_FLOAT32 ||
            (d->ndims == 3 && d->dims[2] != 1 && d->dims[2] != 3 && d->dims[2] != 4)) {
            free(*stages);
            *stages = NULL;
            return 0;
        }
    }
    return 1;
}

static PyObject *mp_gen_finish(PyGPUGeneratorObject *g, PyObject *img)
{
    if (!g->return_to_host) return img;
    PyObject *h = PyGPUArray_to_array((PyGPUArrayObject *)img, NULL);
    Py_DECREF(img);
    return h;
}

/* Reference path: clone inputs[i % n], run each Operation (src/gpugenerator.c:202-281). */
static PyObject *mp_gen_one(PyGPUGeneratorObject *g, long i)
{
    Py_ssize_t n = PyList_GET_SIZE(g->inputs);
    PyObject *src = PyList_GET_ITEM(g->inputs, i % n);
    PyObject *img = PyObject_CallMethod(src, "clone", NULL);
    if (!img) return NULL;
    for (Py_ssize_t k = 0; k < PyList_GET_SIZE(g->operations); ++k) {
        PyGPUOperationObject *op = (PyGPUOperationObject *)PyList_GET_ITEM(g->operations, k);
        PyObject *r = op->requires_instance ? PyGPUOperation_run_on(op, img) : PyGPUOperation_run(op, NULL);
        if (!r) { Py_DECREF(img); return NULL; }
        Py_DECREF(r);
    }
    return mp_gen_finish(g, img);
}

static int mp_gen_fill(PyGPUGeneratorObject *g, MPStage *stages, int nst)
{
    Py_ssize_t n = PyList_GET_SIZE(g->inputs);
    long count = MP_GEN_BATCH;
    if (g->max != NO_OUTPUT_MAX && g->max - g->i < count) count = g->max - g->i;
    /* bound the batch's output bytes */
    unsigned long long bytes = 0;
    long c = 0;
    for (; c < count; ++c) {
        MPObjData *d = ((PyGPUArrayObject *)PyList_GET_ITEM(g->inputs, (g->i + c) % n))->obj_data;
        bytes += d->nbytes;
        if (c > 0 && bytes > MP_GEN_BATCH_BYTES) break;
    }
    count = c;
    MPObjData **srcs = (MPObjData **)malloc(sizeof(MPObjData *) * (size_t)count);
    MPObjData **outs = (MPObjData **)calloc((size_t)count, sizeof(MPObjData *));
    if (!srcs || !outs) { free(srcs); free(outs); PyErr_NoMemory(); return -1; }
    for (long k = 0; k < count; ++k) {
        srcs[k] = ((PyGPUArrayObject *)PyList_GET_ITEM(g->inputs, (g->i + k) % n))->obj_data;
        outs[k] = (MPObjData *)calloc(1, sizeof(MPObjData));
        if (!outs[k]) {
            for (long q = 0; q < k; ++q) free(outs[q]);
            free(srcs); free(outs); PyErr_NoMemory(); return -1;
        }
    }
    MPStatus st;
    Py_BEGIN_ALLOW_THREADS
    st = mpk_pipeline_produce(stages, nst, srcs, outs, (int)count, g->seed, (uint64_t)g->i);
    Py_END_ALLOW_THREADS
    free(srcs);
    if (st != MILLIPYDE_SUCCESS) {
        for (long k = 0; k < count; ++k) free(outs[k]);
        free(outs);
        mp_raise(st);
        return -1;
    }
    int rc = 0;
    for (long k = 0; k < count; ++k) {
        PyObject *img = mp_wrap_obj(&PyGPUImage_Type, outs[k]);   /* steals outs[k] */
        if (!img || PyList_Append(g->ready, img) < 0) rc = -1;
        Py_XDECREF(img);
    }
    free(outs);
    return rc;
}

static PyObject *PyGPUGenerator_next(PyGPUGeneratorObject *g)
{
    if (!g->inputs || !g->operations) return NULL;
    if (g->max != NO_OUTPUT_MAX && g->i >= g->max) {
        Py_CLEAR(g->inputs);
        Py_CLEAR(g->operations);
        return NULL;   /* StopIteration */
    }
    if (PyList_GET_SIZE(g->inputs) == 0) {
        PyErr_SetString(PyExc_ValueError, mperr_str(GPUGENERATOR_ERROR_INVALID_INPUT));
        return NULL;
    }
    if (PyList_GET_SIZE(g->ready) == 0) {
        MPStage *stages;
        int nst;
        int b = mp_gen_batchable(g, &stages, &nst);
        if (b < 0) return NULL;
        if (b == 0) {
            PyObject *r = mp_gen_one(g, g->i);
            if (r) g->i++;
            return r;
        }
        int rc = mp_gen_fill(g, stages, nst);
        free(stages);
        if (rc < 0) return NULL;
    }
    PyObject *img = PyList_GET_ITEM(g->ready, 0);
    Py_INCREF(img);
    if (PySequence_DelItem(g->ready, 0) < 0) { Py_DECREF(img); return NULL; }
    g->i++;
    return mp_gen_finish(g, img);
}

static PyMemberDef PyGPUGenerator_members[] = {
    {"seed", T_ULONGLONG, offsetof(PyGPUGeneratorObject, seed), READONLY,
     "seed of the counter RNG the batched path draws random parameters from"},
    {NULL}};

PyTypeObject PyGPUGenerator_Type = {
    PyVarObject_HEAD_INIT(NULL, 0).tp_name = "millipyde.Generator",
    .tp_basicsize = sizeof(PyGPUGeneratorObject),
    .tp_dealloc = (destructor)PyGPUGenerator_dealloc,
    .tp_flags = Py_TPFLAGS_DEFAULT,
    .tp_doc = "Generator(inputs_or_path, operations, device=, outputs=, return_to_host=, seed=)",
    .tp_iter = PyGPUGenerator_iter,
    .tp_iternext = (iternextfunc)PyGPUGenerator_next,
    .tp_members = PyGPUGenerator_members,
    .tp_init = (initproc)PyGPUGenerator_init,
    .tp_new = PyGPUGenerator_new,
};

/* ======================================================================== */
/* Device                                                                   */
/* ======================================================================== */
static int PyDevice_init(PyDeviceObject *self, PyObject *args, PyObject *kwds)
{
    int d;
    if (!PyArg_ParseTuple(args, "i", &d)) return -1;
    self->device_id = d;
    self->prev_device_id = DEVICE_LOC_NO_AFFINITY;
    return 0;
}

static PyObject *PyDevice_enter(PyDeviceObject *self, PyObject *unused)
{
    if (!mpdev_is_valid_device(self->device_id)) {
        PyErr_SetString(PyExc_ValueError, mperr_str(DEV_WARN_BAD_DEVICE));
        return NULL;
    }
    self->prev_device_id = mpdev_get_target_device();
    mpdev_set_target_device(self->device_id);
    return PyLong_FromLong(self->device_id);
}

/* Restores the previous target device; an exception propagates unchanged
 * (the reference reset the whole device here, src/device.c:60-64). */
static PyObject *PyDevice_exit(PyDeviceObject *self, PyObject *args)
{
    PyObject *et, *ev, *tb;
    if (!PyArg_ParseTuple(args, "OOO", &et, &ev, &tb)) return NULL;
    MPStatus st = MILLIPYDE_SUCCESS;
    if (et == Py_None) {
        Py_BEGIN_ALLOW_THREADS
        st = mpdev_synchronize();
        Py_END_ALLOW_THREADS
    }
    mpdev_set_target_device(self->prev_device_id);
    if (st != MILLIPYDE_SUCCESS && st != MP_ERROR_NO_DEVICE) return mp_raise(st);
    Py_RETURN_FALSE;
}

static PyMethodDef PyDevice_methods[] = {
    {"__enter__", (PyCFunction)PyDevice_enter, METH_NOARGS, "Make this the target device."},
    {"__exit__", (PyCFunction)PyDevice_exit, METH_VARARGS, "Restore the previous target device."},
    {NULL}};

PyTypeObject PyDevice_Type = {
    PyVarObject_HEAD_INIT(NULL, 0).tp_name = "millipyde.Device",
    .tp_basicsize = sizeof(PyDeviceObject),
    .tp_flags = Py_TPFLAGS_DEFAULT,
    .tp_doc = "Device(id): context manager that sets the target GPU.",
    .tp_methods = PyDevice_methods,
    .tp_init = (initproc)PyDevice_init,
    .tp_new = PyType_GenericNew,
};
