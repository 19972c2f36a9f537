/*
 * py_objects.c -- the gpuarray and gpuimage types.
 *
 * gpuarray  (reference src/gpuarray.c): a numeric array resident on the GPU;
 *           np.array(x) copies it back; clone(); NumPy protocol fallbacks.
 * gpuimage  (reference src/gpuimage.c): a 2-D (greyscale) or 3-D
 *           (height, width, channels) gpuarray with in-place image methods.
 *           Rows are stored with a 16-byte-aligned pitch on the device.
 * Methods mutate the image in place and return None, as in the reference.
 */
#include "py_common.h"

#include <math.h>

/* ------------------------------------------------------------------------ */
/* errors                                                                    */
/* ------------------------------------------------------------------------ */
PyObject *mp_raise(MPStatus st)
{
    PyObject *exc = PyExc_RuntimeError;
    switch (st) {
    case MP_ERROR_INVALID_ARGS:
    case MP_ERROR_TOO_LARGE:
    case MP_ERROR_UNSUPPORTED_DIMS:
    case MP_ERROR_BAD_DESCRIPTOR: exc = PyExc_ValueError; break;
    case MP_ERROR_UNSUPPORTED_TYPE: exc = PyExc_TypeError; break;
    case MP_ERROR_OUT_OF_MEMORY: exc = PyExc_MemoryError; break;
    default: break;
    }
    const char *cuda = mp_last_cuda_error();
    if ((st == MP_ERROR_CUDA || st == MP_ERROR_NO_DEVICE || st == MP_ERROR_OUT_OF_MEMORY) && cuda && cuda[0])
        PyErr_Format(exc, "%s (%s)", mperr_str(st), cuda);
    else
        PyErr_SetString(exc, mperr_str(st));
    return NULL;
}

int mp_raise_int(MPStatus st)
{
    mp_raise(st);
    return -1;
}

/* ------------------------------------------------------------------------ */
/* gpuarray                                                                  */
/* ------------------------------------------------------------------------ */
int mp_is_gpuarray(PyObject *o) { return PyObject_TypeCheck(o, &PyGPUArray_Type); }
int mp_is_gpuimage(PyObject *o) { return PyObject_TypeCheck(o, &PyGPUImage_Type); }

static void PyGPUArray_dealloc(PyGPUArrayObject *self)
{
    if (self->obj_data) {
        mpobj_dealloc_device_data(self->obj_data);
        free(self->obj_data);
        self->obj_data = NULL;
    }
    Py_XDECREF(self->array_data);
    Py_TYPE(self)->tp_free((PyObject *)self);
}

static PyObject *PyGPUArray_new(PyTypeObject *type, PyObject *args, PyObject *kwds)
{
    PyGPUArrayObject *self = (PyGPUArrayObject *)type->tp_alloc(type, 0);
    if (self) {
        self->array_data = NULL;
        self->obj_data = NULL;
    }
    return (PyObject *)self;
}

/* Converts `any` to a C-contiguous numeric ndarray (new reference) or sets
 * ValueError with the given status. */
static PyArrayObject *mp_as_numeric_array(PyObject *any, MPStatus not_array, MPStatus not_numeric)
{
    if (any == NULL || any == Py_None) {
        PyErr_SetString(PyExc_ValueError, mperr_str(not_array));
        return NULL;
    }
    PyArrayObject *arr =
        (PyArrayObject *)PyArray_FROM_OTF(any, NPY_NOTYPE, NPY_ARRAY_IN_ARRAY | NPY_ARRAY_ENSUREARRAY);
    if (!arr) {
        PyErr_Clear();
        PyErr_SetString(PyExc_ValueError, mperr_str(not_array));
        return NULL;
    }
    if (!PyArray_ISNUMBER(arr)) {
        Py_DECREF(arr);
        PyErr_SetString(PyExc_ValueError, mperr_str(not_numeric));
        return NULL;
    }
    return arr;
}

static int mp_init_from_array(PyGPUArrayObject *self, PyArrayObject *arr, int image)
{
    int nd = PyArray_NDIM(arr);
    int64_t shape[32];
    for (int i = 0; i < nd; ++i) shape[i] = (int64_t)PyArray_DIM(arr, i);
    MPObjData *obj = (MPObjData *)calloc(1, sizeof(MPObjData));
    if (!obj) {
        PyErr_NoMemory();
        return -1;
    }
    MPStatus st;
    Py_BEGIN_ALLOW_THREADS
    st = mpobj_copy_from_host(obj, PyArray_DATA(arr), nd, shape, PyArray_TYPE(arr),
                              (int)PyArray_ITEMSIZE(arr), image ? MP_TRUE : MP_FALSE);
    Py_END_ALLOW_THREADS
    if (st != MILLIPYDE_SUCCESS) {
        free(obj);
        return mp_raise_int(st);
    }
    if (self->obj_data) {
        mpobj_dealloc_device_data(self->obj_data);
        free(self->obj_data);
    }
    self->obj_data = obj;
    return 0;
}

static int PyGPUArray_init(PyGPUArrayObject *self, PyObject *args, PyObject *kwds)
{
    PyObject *any = NULL;
    if (!PyArg_ParseTuple(args, "O", &any)) return -1;
    PyArrayObject *arr = mp_as_numeric_array(any, GPUARRAY_ERROR_CONSTRUCTION_WITHOUT_ARRAY_TYPE,
                                             GPUARRAY_ERROR_CONSTRUCTION_WITHOUT_NUMERIC_ARRAY);
    if (!arr) return -1;
    int r = mp_init_from_array(self, arr, 0);
    Py_DECREF(arr);
    return r;
}

PyObject *PyGPUArray_to_array(PyGPUArrayObject *self, PyObject *unused)
{
    MPObjData *o = self->obj_data;
    if (!o) {
        PyErr_SetString(PyExc_ValueError, "gpuarray has no data");
        return NULL;
    }
    npy_intp dims[32];
    for (int i = 0; i < o->ndims; ++i) dims[i] = o->dims[i];
    PyObject *arr = PyArray_SimpleNew(o->ndims, dims, o->type);
    if (!arr) return NULL;
    MPStatus st;
    void *dst = PyArray_DATA((PyArrayObject *)arr);
    Py_BEGIN_ALLOW_THREADS
    st = mpobj_copy_to_host(o, dst);
    Py_END_ALLOW_THREADS
    if (st != MILLIPYDE_SUCCESS) {
        Py_DECREF(arr);
        return mp_raise(st);
    }
    return arr;
}

/* __array__(dtype=None, copy=None) */
static PyObject *PyGPUArray_array(PyGPUArrayObject *self, PyObject *args, PyObject *kwds)
{
    static char *kwlist[] = {"dtype", "copy", NULL};
    PyObject *dtype = Py_None, *copy = Py_None;
    if (!PyArg_ParseTupleAndKeywords(args, kwds, "|OO", kwlist, &dtype, &copy)) return NULL;
    PyObject *arr = PyGPUArray_to_array(self, NULL);
    if (!arr || dtype == Py_None) return arr;
    PyObject *res = PyObject_CallMethod(arr, "astype", "O", dtype);
    Py_DECREF(arr);
    return res;
}

/* Replaces gpuarray arguments by host ndarrays, one level into lists/tuples. */
static PyObject *mp_to_host_arg(PyObject *a)
{
    if (mp_is_gpuarray(a)) return PyGPUArray_to_array((PyGPUArrayObject *)a, NULL);
    if (PyList_Check(a) || PyTuple_Check(a)) {
        Py_ssize_t n = PySequence_Size(a);
        PyObject *lst = PyList_New(n);
        if (!lst) return NULL;
        for (Py_ssize_t i = 0; i < n; ++i) {
            PyObject *it = PySequence_GetItem(a, i);
            if (!it) { Py_DECREF(lst); return NULL; }
            PyObject *c = mp_is_gpuarray(it) ? PyGPUArray_to_array((PyGPUArrayObject *)it, NULL) : (Py_INCREF(it), it);
            Py_DECREF(it);
            if (!c) { Py_DECREF(lst); return NULL; }
            PyList_SET_ITEM(lst, i, c);
        }
        if (PyTuple_Check(a)) {
            PyObject *t = PyList_AsTuple(lst);
            Py_DECREF(lst);
            return t;
        }
        return lst;
    }
    Py_INCREF(a);
    return a;
}

static PyObject *mp_to_host_tuple(PyObject *tup)
{
    Py_ssize_t n = PyTuple_Size(tup);
    PyObject *out = PyTuple_New(n);
    if (!out) return NULL;
    for (Py_ssize_t i = 0; i < n; ++i) {
        PyObject *c = mp_to_host_arg(PyTuple_GET_ITEM(tup, i));
        if (!c) { Py_DECREF(out); return NULL; }
        PyTuple_SET_ITEM(out, i, c);
    }
    return out;
}

static PyObject *mp_to_host_dict(PyObject *d)
{
    if (!d || d == Py_None) return PyDict_New();
    PyObject *out = PyDict_New();
    PyObject *k, *v;
    Py_ssize_t pos = 0;
    while (PyDict_Next(d, &pos, &k, &v)) {
        PyObject *c = mp_to_host_arg(v);
        if (!c || PyDict_SetItem(out, k, c) < 0) { Py_XDECREF(c); Py_DECREF(out); return NULL; }
        Py_DECREF(c);
    }
    return out;
}

/* __array_function__(func, types, args, kwargs): host fallback
 * (reference src/gpuarray.c:193-226). */
static PyObject *PyGPUArray_array_function(PyGPUArrayObject *self, PyObject *args)
{
    PyObject *func, *types, *fargs, *fkw;
    if (!PyArg_ParseTuple(args, "OOOO", &func, &types, &fargs, &fkw)) return NULL;
    PyObject *hargs = mp_to_host_tuple(fargs);
    if (!hargs) return NULL;
    PyObject *hkw = mp_to_host_dict(fkw);
    if (!hkw) { Py_DECREF(hargs); return NULL; }
    PyObject *res = PyObject_Call(func, hargs, hkw);
    Py_DECREF(hargs);
    Py_DECREF(hkw);
    return res;
}

/* __array_ufunc__(ufunc, method, *inputs, **kwargs): host fallback; the
 * reference's version (src/gpuarray.c:146-191) printed debug text and passed
 * the wrong arguments. */
static PyObject *PyGPUArray_array_ufunc(PyGPUArrayObject *self, PyObject *args, PyObject *kwds)
{
    Py_ssize_t n = PyTuple_Size(args);
    if (n < 2) {
        PyErr_SetString(PyExc_TypeError, "__array_ufunc__ needs (ufunc, method, *inputs)");
        return NULL;
    }
    PyObject *ufunc = PyTuple_GET_ITEM(args, 0);
    PyObject *method = PyTuple_GET_ITEM(args, 1);
    if (kwds && PyDict_GetItemString(kwds, "out")) {
        PyObject *outs = PyDict_GetItemString(kwds, "out");
        PyObject *seq = PySequence_Fast(outs, "out");
        if (!seq) return NULL;
        for (Py_ssize_t i = 0; i < PySequence_Fast_GET_SIZE(seq); ++i) {
            if (mp_is_gpuarray(PySequence_Fast_GET_ITEM(seq, i))) {
                Py_DECREF(seq);
                Py_RETURN_NOTIMPLEMENTED;
            }
        }
        Py_DECREF(seq);
    }
    PyObject *inputs = PyTuple_GetSlice(args, 2, n);
    if (!inputs) return NULL;
    PyObject *hin = mp_to_host_tuple(inputs);
    Py_DECREF(inputs);
    if (!hin) return NULL;
    PyObject *hkw = mp_to_host_dict(kwds);
    if (!hkw) { Py_DECREF(hin); return NULL; }
    PyObject *fn = PyObject_GetAttr(ufunc, method);
    PyObject *res = fn ? PyObject_Call(fn, hin, hkw) : NULL;
    Py_XDECREF(fn);
    Py_DECREF(hin);
    Py_DECREF(hkw);
    return res;
}

PyObject *mp_wrap_obj(PyTypeObject *type, MPObjData *obj)
{
    PyGPUArrayObject *o = (PyGPUArrayObject *)type->tp_alloc(type, 0);
    if (!o) {
        mpobj_dealloc_device_data(obj);
        free(obj);
        return NULL;
    }
    o->array_data = NULL;
    o->obj_data = obj;
    if (PyType_IsSubtype(type, &PyGPUImage_Type)) {
        ((PyGPUImageObject *)o)->height = obj->ndims >= 1 ? obj->dims[0] : 0;
        ((PyGPUImageObject *)o)->width = obj->ndims >= 2 ? obj->dims[1] : 0;
    }
    return (PyObject *)o;
}

static PyObject *PyGPUArray_clone(PyGPUArrayObject *self, PyObject *unused)
{
    if (!self->obj_data) {
        PyErr_SetString(PyExc_ValueError, "gpuarray has no data");
        return NULL;
    }
    MPObjData *c = mpobj_clone_data(self->obj_data, self->obj_data->mem_loc, 0);
    if (!c) return mp_raise(MP_ERROR_CUDA);
    return mp_wrap_obj(Py_TYPE(self), c);
}

static PyObject *PyGPUArray_get_shape(PyGPUArrayObject *self, void *closure)
{
    MPObjData *o = self->obj_data;
    if (!o) Py_RETURN_NONE;
    PyObject *t = PyTuple_New(o->ndims);
    for (int i = 0; i < o->ndims; ++i) PyTuple_SET_ITEM(t, i, PyLong_FromLong(o->dims[i]));
    return t;
}

static PyObject *PyGPUArray_get_dtype(PyGPUArrayObject *self, void *closure)
{
    if (!self->obj_data) Py_RETURN_NONE;
    PyArray_Descr *d = PyArray_DescrFromType(self->obj_data->type);
    return (PyObject *)d;
}

static PyObject *PyGPUArray_get_ndim(PyGPUArrayObject *self, void *closure)
{
    return PyLong_FromLong(self->obj_data ? self->obj_data->ndims : 0);
}

static PyMethodDef PyGPUArray_methods[] = {
    {"__array__", (PyCFunction)PyGPUArray_array, METH_VARARGS | METH_KEYWORDS,
     "Copy the array back to the host as a numpy.ndarray."},
    {"__array_function__", (PyCFunction)PyGPUArray_array_function, METH_VARARGS,
     "NumPy function protocol: runs the function on host copies."},
    {"__array_ufunc__", (PyCFunction)PyGPUArray_array_ufunc, METH_VARARGS | METH_KEYWORDS,
     "NumPy ufunc protocol: runs the ufunc on host copies."},
    {"clone", (PyCFunction)PyGPUArray_clone, METH_NOARGS, "Deep copy on the same device."},
    {NULL}};

static PyGetSetDef PyGPUArray_getset[] = {
    {"shape", (getter)PyGPUArray_get_shape, NULL, "array shape", NULL},
    {"dtype", (getter)PyGPUArray_get_dtype, NULL, "element type", NULL},
    {"ndim", (getter)PyGPUArray_get_ndim, NULL, "number of dimensions", NULL},
    {NULL}};

PyTypeObject PyGPUArray_Type = {
    PyVarObject_HEAD_INIT(NULL, 0).tp_name = "millipyde.gpuarray",
    .tp_basicsize = sizeof(PyGPUArrayObject),
    .tp_dealloc = (destructor)PyGPUArray_dealloc,
    .tp_flags = Py_TPFLAGS_DEFAULT | Py_TPFLAGS_BASETYPE,
    .tp_doc = "A numeric array resident in GPU memory.",
    .tp_methods = PyGPUArray_methods,
    .tp_getset = PyGPUArray_getset,
    .tp_init = (initproc)PyGPUArray_init,
    .tp_new = PyGPUArray_new,
};

/* ------------------------------------------------------------------------ */
/* gpuimage                                                                  */
/* ------------------------------------------------------------------------ */
static int PyGPUImage_init(PyGPUImageObject *self, PyObject *args, PyObject *kwds)
{
    PyObject *any = NULL;
    if (!PyArg_ParseTuple(args, "O", &any)) return -1;
    PyArrayObject *arr = mp_as_numeric_array(any, GPUIMAGE_ERROR_CONSTRUCTION_WITHOUT_ARRAY_TYPE,
                                             GPUIMAGE_ERROR_CONSTRUCTION_WITHOUT_IMAGE_FORMAT);
    if (!arr) return -1;
    int nd = PyArray_NDIM(arr);
    if (nd != 2 && nd != 3) {
        Py_DECREF(arr);
        PyErr_SetString(PyExc_ValueError, mperr_str(GPUIMAGE_ERROR_CONSTRUCTION_WITHOUT_IMAGE_DIMS));
        return -1;
    }
    int r = mp_init_from_array(&self->array, arr, 1);
    Py_DECREF(arr);
    if (r < 0) return -1;
    self->height = self->array.obj_data->dims[0];
    self->width = self->array.obj_data->dims[1];
    return 0;
}

static MPObjData *mp_img(PyGPUImageObject *self)
{
    if (!self->array.obj_data) PyErr_SetString(PyExc_ValueError, "gpuimage has no data");
    return self->array.obj_data;
}

/* Runs one C-ABI op on the image without the GIL; None or an exception. */
static PyObject *mp_run_op(PyGPUImageObject *self, MPFunc fn, void *args)
{
    MPObjData *o = mp_img(self);
    if (!o) return NULL;
    MPStatus st;
    Py_BEGIN_ALLOW_THREADS
    st = fn(o, args);
    Py_END_ALLOW_THREADS
    if (st != MILLIPYDE_SUCCESS) return mp_raise(st);
    self->height = o->dims[0];
    self->width = o->dims[1];
    Py_RETURN_NONE;
}

static PyObject *PyGPUImage_color_to_greyscale(PyGPUImageObject *self, PyObject *unused)
{
    return mp_run_op(self, mpimg_color_to_greyscale, NULL);
}

static PyObject *PyGPUImage_transpose(PyGPUImageObject *self, PyObject *unused)
{
    return mp_run_op(self, mpimg_transpose, NULL);
}

static PyObject *PyGPUImage_fliplr(PyGPUImageObject *self, PyObject *unused)
{
    return mp_run_op(self, mpimg_fliplr, NULL);
}

static PyObject *PyGPUImage_rotate(PyGPUImageObject *self, PyObject *args)
{
    RotateArgs a;
    if (!PyArg_ParseTuple(args, "d", &a.angle)) return NULL;
    return mp_run_op(self, mpimg_rotate, &a);
}

static PyObject *PyGPUImage_gaussian(PyGPUImageObject *self, PyObject *args)
{
    GaussianArgs a;
    if (!PyArg_ParseTuple(args, "d", &a.sigma)) return NULL;
    if (!(a.sigma > 0.0)) {
        PyErr_SetString(PyExc_ValueError, "gaussian sigma must be positive");
        return NULL;
    }
    return mp_run_op(self, mpimg_gaussian, &a);
}

/* src/gpuimage.c:719-737: delta must lie strictly inside (-1, 1). */
static PyObject *PyGPUImage_brightness(PyGPUImageObject *self, PyObject *args)
{
    BrightnessArgs a;
    if (!PyArg_ParseTuple(args, "d", &a.delta)) return NULL;
    if (a.delta <= -1.0 || a.delta >= 1.0) {
        PyErr_SetString(PyExc_ValueError, "brightness delta must lie strictly between -1 and 1");
        return NULL;
    }
    return mp_run_op(self, mpimg_brightness, &a);
}

/* adjust_gamma(gamma, gain=1); the reference required gain (src/gpuimage.c:765-781). */
static PyObject *PyGPUImage_adjust_gamma(PyGPUImageObject *self, PyObject *args)
{
    GammaArgs a;
    a.gain = 1.0;
    if (!PyArg_ParseTuple(args, "d|d", &a.gamma, &a.gain)) return NULL;
    return mp_run_op(self, mpimg_adjust_gamma, &a);
}

static PyObject *PyGPUImage_colorize(PyGPUImageObject *self, PyObject *args)
{
    ColorizeArgs a;
    if (!PyArg_ParseTuple(args, "ddd", &a.r_mult, &a.g_mult, &a.b_mult)) return NULL;
    if (a.r_mult < 0 || a.g_mult < 0 || a.b_mult < 0) {
        PyErr_SetString(PyExc_ValueError, "colorize multipliers must be non-negative");
        return NULL;
    }
    return mp_run_op(self, mpimg_colorize, &a);
}

static int mp_draw(double lo, double hi, double *out)
{
    if (random_double_in_range(lo, hi, out) != MILLIPYDE_SUCCESS) {
        PyErr_SetString(PyExc_RuntimeError, mperr_str(RAND_ERROR_INSUFFICIENT_BYTES));
        return -1;
    }
    return 0;
}

/* Reads a [lo, hi] pair from a list/tuple. */
static int mp_range(PyObject *o, double *lo, double *hi)
{
    PyObject *seq = PySequence_Fast(o, "expected a [min, max] list");
    if (!seq) return -1;
    if (PySequence_Fast_GET_SIZE(seq) != 2) {
        Py_DECREF(seq);
        PyErr_SetString(PyExc_ValueError, "expected a [min, max] list");
        return -1;
    }
    *lo = PyFloat_AsDouble(PySequence_Fast_GET_ITEM(seq, 0));
    *hi = PyFloat_AsDouble(PySequence_Fast_GET_ITEM(seq, 1));
    Py_DECREF(seq);
    return PyErr_Occurred() ? -1 : 0;
}

static PyObject *PyGPUImage_rand_rotate(PyGPUImageObject *self, PyObject *args)
{
    double lo, hi;
    RotateArgs a;
    if (!PyArg_ParseTuple(args, "dd", &lo, &hi)) return NULL;
    if (mp_draw(lo, hi, &a.angle) < 0) return NULL;
    return mp_run_op(self, mpimg_rotate, &a);
}

static PyObject *PyGPUImage_rand_gaussian(PyGPUImageObject *self, PyObject *args)
{
    double lo, hi;
    GaussianArgs a;
    if (!PyArg_ParseTuple(args, "dd", &lo, &hi)) return NULL;
    if (mp_draw(lo, hi, &a.sigma) < 0) return NULL;
    if (!(a.sigma > 0.0)) {
        PyErr_SetString(PyExc_ValueError, "gaussian sigma must be positive");
        return NULL;
    }
    return mp_run_op(self, mpimg_gaussian, &a);
}

static PyObject *PyGPUImage_rand_brightness(PyGPUImageObject *self, PyObject *args)
{
    double lo, hi;
    BrightnessArgs a;
    if (!PyArg_ParseTuple(args, "dd", &lo, &hi)) return NULL;
    if (mp_draw(lo, hi, &a.delta) < 0) return NULL;
    return mp_run_op(self, mpimg_brightness, &a);
}

/* random_adjust_gamma([gmin, gmax], [gain_min, gain_max]) as in the reference
 * (src/gpuimage.c:397-432), or random_adjust_gamma(gmin, gmax) with gain 1. */
static PyObject *PyGPUImage_rand_adjust_gamma(PyGPUImageObject *self, PyObject *args)
{
    PyObject *a0, *a1;
    GammaArgs a;
    if (!PyArg_ParseTuple(args, "OO", &a0, &a1)) return NULL;
    if (PySequence_Check(a0) && PySequence_Check(a1)) {
        double g0, g1, k0, k1;
        if (mp_range(a0, &g0, &g1) < 0 || mp_range(a1, &k0, &k1) < 0) return NULL;
        if (mp_draw(g0, g1, &a.gamma) < 0 || mp_draw(k0, k1, &a.gain) < 0) return NULL;
    } else {
        double g0 = PyFloat_AsDouble(a0), g1 = PyFloat_AsDouble(a1);
        if (PyErr_Occurred()) return NULL;
        if (mp_draw(g0, g1, &a.gamma) < 0) return NULL;
        a.gain = 1.0;
    }
    return mp_run_op(self, mpimg_adjust_gamma, &a);
}

static PyObject *PyGPUImage_rand_colorize(PyGPUImageObject *self, PyObject *args)
{
    PyObject *r, *g, *b;
    ColorizeArgs a;
    double lo, hi;
    if (!PyArg_ParseTuple(args, "OOO", &r, &g, &b)) return NULL;
    if (mp_range(r, &lo, &hi) < 0 || mp_draw(lo, hi, &a.r_mult) < 0) return NULL;
    if (mp_range(g, &lo, &hi) < 0 || mp_draw(lo, hi, &a.g_mult) < 0) return NULL;
    if (mp_range(b, &lo, &hi) < 0 || mp_draw(lo, hi, &a.b_mult) < 0) return NULL;
    if (a.r_mult < 0 || a.g_mult < 0 || a.b_mult < 0) {
        PyErr_SetString(PyExc_ValueError, "colorize multipliers must be non-negative");
        return NULL;
    }
    return mp_run_op(self, mpimg_colorize, &a);
}

static PyMethodDef PyGPUImage_methods[] = {
    {"rgb2gray", (PyCFunction)PyGPUImage_color_to_greyscale, METH_NOARGS, "Convert to greyscale in place."},
    {"rgb2grey", (PyCFunction)PyGPUImage_color_to_greyscale, METH_NOARGS, "Convert to greyscale in place."},
    {"rgba2gray", (PyCFunction)PyGPUImage_color_to_greyscale, METH_NOARGS, "Convert to greyscale in place."},
    {"rgba2grey", (PyCFunction)PyGPUImage_color_to_greyscale, METH_NOARGS, "Convert to greyscale in place."},
    {"transpose", (PyCFunction)PyGPUImage_transpose, METH_NOARGS, "Swap rows and columns in place."},
    {"gaussian", (PyCFunction)PyGPUImage_gaussian, METH_VARARGS,
     "gaussian(sigma): zero-padded gaussian blur, radius ceil(3*sigma)."},
    {"random_gaussian", (PyCFunction)PyGPUImage_rand_gaussian, METH_VARARGS,
     "random_gaussian(min, max): gaussian with sigma drawn uniformly."},
    {"brightness", (PyCFunction)PyGPUImage_brightness, METH_VARARGS,
     "brightness(delta): add delta, clamp to [0, 1]."},
    {"random_brightness", (PyCFunction)PyGPUImage_rand_brightness, METH_VARARGS,
     "random_brightness(min, max)."},
    {"adjust_gamma", (PyCFunction)PyGPUImage_adjust_gamma, METH_VARARGS,
     "adjust_gamma(gamma, gain=1): gain * x**gamma clamped to [0, 1]."},
    {"random_adjust_gamma", (PyCFunction)PyGPUImage_rand_adjust_gamma, METH_VARARGS,
     "random_adjust_gamma([gmin, gmax], [gain_min, gain_max]) or (gmin, gmax)."},
    {"colorize", (PyCFunction)PyGPUImage_colorize, METH_VARARGS,
     "colorize(r, g, b): scale colour channels, clamp to 1."},
    {"random_colorize", (PyCFunction)PyGPUImage_rand_colorize, METH_VARARGS,
     "random_colorize([r0, r1], [g0, g1], [b0, b1])."},
    {"fliplr", (PyCFunction)PyGPUImage_fliplr, METH_NOARGS, "Mirror left-right in place."},
    {"rotate", (PyCFunction)PyGPUImage_rotate, METH_VARARGS,
     "rotate(angle): bilinear rotation in degrees about the centre, zero fill."},
    {"random_rotate", (PyCFunction)PyGPUImage_rand_rotate, METH_VARARGS, "random_rotate(min, max)."},
    {NULL}};

static PyMemberDef PyGPUImage_members[] = {
    {"width", T_INT, offsetof(PyGPUImageObject, width), READONLY, "image width"},
    {"height", T_INT, offsetof(PyGPUImageObject, height), READONLY, "image height"},
    {NULL}};

PyTypeObject PyGPUImage_Type = {
    PyVarObject_HEAD_INIT(NULL, 0).tp_name = "millipyde.gpuimage",
    .tp_basicsize = sizeof(PyGPUImageObject),
    .tp_flags = Py_TPFLAGS_DEFAULT | Py_TPFLAGS_BASETYPE,
    .tp_doc = "An image resident in GPU memory: (height, width) or (height, width, channels).",
    .tp_methods = PyGPUImage_methods,
    .tp_members = PyGPUImage_members,
    .tp_init = (initproc)PyGPUImage_init,
};
