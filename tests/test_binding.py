"""Host-side logic of the Python binding (no GPU)."""
import weakref

import vlb


class _Rec:
    def __init__(self, log, name):
        self.log, self.name = log, name

    def close(self):
        self.log.append(self.name)


def test_context_close_destroys_services_first(monkeypatch):
    """A service's destroy joins its worker, which may still be baking with
    the scenes, direction sets and skies its requests name: Context.close()
    closes every service before any other object, then the context."""
    log = []

    class FakeService(vlb.Service, _Rec):
        def __init__(self, name):
            _Rec.__init__(self, log, name)

        close = _Rec.close

    class FakeScene(_Rec):
        pass

    ctx = vlb.Context.__new__(vlb.Context)
    ctx.h = object()
    ctx._objects = weakref.WeakSet()
    objs = [FakeScene(log, "scene0"), FakeService("svc0"), FakeScene(log, "dirs0"), FakeService("svc1"),
            FakeScene(log, "sky0")]
    for o in objs:
        ctx._own(o)
    monkeypatch.setattr(vlb.lib, "vlb_ctx_destroy", lambda h: log.append("ctx"))
    ctx.close()
    assert sorted(log[:2]) == ["svc0", "svc1"]
    assert sorted(log[2:5]) == ["dirs0", "scene0", "sky0"]
    assert log[5:] == ["ctx"] and ctx.h is None
