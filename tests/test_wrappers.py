"""Host logic of the Python wrappers (no device): closing a context destroys
the scenes and models made on it first, once, whatever order their own
close() or finalizers run in afterwards."""
import ctypes

from risltc_gb300 import api


class FakeLib:
    def __init__(self):
        self.calls = []

    def risltc_ctx_destroy(self, h):
        self.calls.append(("ctx", h.value))

    def risltc_scene_destroy(self, h):
        self.calls.append(("scene", h.value))

    def risltc_model_destroy(self, h):
        self.calls.append(("model", h.value))


def make(lib):
    ctx = api.Context.__new__(api.Context)
    ctx._lib, ctx._h, ctx._owned = lib, ctypes.c_void_p(1), []
    scene = api.Scene.__new__(api.Scene)
    scene._lib, scene._h = lib, ctypes.c_void_p(2)
    ctx._adopt(lib.risltc_scene_destroy, scene._h)
    model = api.Model.__new__(api.Model)
    model._lib, model._h = lib, ctypes.c_void_p(3)
    ctx._adopt(lib.risltc_model_destroy, model._h)
    return ctx, scene, model


def test_closing_the_context_destroys_its_scenes_and_models_first():
    lib = FakeLib()
    ctx, scene, model = make(lib)
    ctx.close()
    assert lib.calls == [("model", 3), ("scene", 2), ("ctx", 1)]
    assert not scene.handle and not model.handle
    scene.close()
    model.close()
    ctx.close()
    assert len(lib.calls) == 3


def test_children_closed_first_are_not_destroyed_again():
    lib = FakeLib()
    ctx, scene, model = make(lib)
    model.close()
    scene.close()
    ctx.close()
    assert lib.calls == [("model", 3), ("scene", 2), ("ctx", 1)]
