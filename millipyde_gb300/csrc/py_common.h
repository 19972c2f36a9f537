/*
 * py_common.h -- declarations shared by the CPython extension's C files.
 *
 * The extension mirrors the reference's Python layer (src/gpuarray.c,
 * src/gpuimage.c, src/gpuoperation.c, src/gpupipeline.c, src/gpugenerator.c,
 * src/device.c, src/millipyde_module.c): same type names, method names,
 * argument meaning and error types, calling the C-ABI in
 * include/millipyde_gb300.h.
 */
#ifndef MP_PY_COMMON_H
#define MP_PY_COMMON_H

#define PY_SSIZE_T_CLEAN
#include <Python.h>
#include <structmember.h>

#define NPY_NO_DEPRECATED_API NPY_1_7_API_VERSION
#define PY_ARRAY_UNIQUE_SYMBOL MP_ARRAY_API
#ifndef MP_MAIN_MODULE
#define NO_IMPORT_ARRAY
#endif
#include <numpy/arrayobject.h>

#include "../../include/millipyde_gb300.h"

typedef struct {
    PyObject_HEAD
    PyObject *array_data;     /* unused; kept for layout parity with the reference */
    MPObjData *obj_data;
} PyGPUArrayObject;

typedef struct {
    PyGPUArrayObject array;
    int width;
    int height;
} PyGPUImageObject;

typedef struct {
    PyObject_HEAD
    PyObject *callable;       /* method name (str) or callable */
    PyObject *arg_tuple;
    MPBool requires_instance;
    double probability;       /* -1: always */
} PyGPUOperationObject;

typedef struct PyGPUPipelineObject {
    PyObject_HEAD
    PyObject *inputs;
    PyObject *operations;
    int device_id;
    struct PyGPUPipelineObject *receiver;
    int has_seed;
    uint64_t seed;
    uint64_t runs;
} PyGPUPipelineObject;

#define NO_OUTPUT_MAX -1

typedef struct {
    PyObject_HEAD
    PyObject *inputs;
    PyObject *operations;
    int device_id;
    long max;
    long i;
    MPBool return_to_host;
    uint64_t seed;
    PyObject *ready;          /* list of produced, not yet returned outputs */
} PyGPUGeneratorObject;

typedef struct {
    PyObject_HEAD
    int device_id;
    int prev_device_id;
} PyDeviceObject;

extern PyTypeObject PyGPUArray_Type;
extern PyTypeObject PyGPUImage_Type;
extern PyTypeObject PyGPUOperation_Type;
extern PyTypeObject PyGPUPipeline_Type;
extern PyTypeObject PyGPUGenerator_Type;
extern PyTypeObject PyDevice_Type;

/* Sets a Python exception for a failed status and returns NULL. */
PyObject *mp_raise(MPStatus st);
/* Same, returning -1 (for tp_init). */
int mp_raise_int(MPStatus st);

/* gpuarray helpers */
PyObject *PyGPUArray_to_array(PyGPUArrayObject *self, PyObject *unused);
int mp_is_gpuarray(PyObject *o);     /* gpuarray or gpuimage (or subclass) */
int mp_is_gpuimage(PyObject *o);
PyObject *mp_wrap_obj(PyTypeObject *type, MPObjData *obj);  /* steals obj */

/* Operation helpers */
MPStatus gpuoperation_evaluate_probability(MPBool *result, double probability);
PyObject *PyGPUOperation_run(PyGPUOperationObject *self, PyObject *unused);
PyObject *PyGPUOperation_run_on(PyGPUOperationObject *self, PyObject *instance);
/* Fills *stage from an Operation built from a method name; returns 1 if the
 * name is a batchable image op, 0 if not (stage untouched), -1 with a Python
 * error set on bad arguments. */
int mp_stage_from_operation(PyGPUOperationObject *op, MPStage *stage);

#endif
