"""The lifecycle entry points of the Python API (crtmv3_gb300/api.py) on a
stand-in library handle: CRTM_Init, CRTM_IsInitialized and CRTM_Destroy
(src/CRTM_LifeCycle.f90:520, :1131, :1291)."""
from crtmv3_gb300 import api


def test_is_initialized_follows_init_and_destroy(coeff_dir, monkeypatch):
    """CRTM_IsInitialized (src/CRTM_LifeCycle.f90:1291-1295) after CRTM_Init and
    CRTM_Destroy, on a stand-in handle."""
    class FakeCRTM:
        def __init__(self, ids, path, *a):
            self.h = object()
            self.n_channels = [22]

        def close(self):
            self.h = None

    monkeypatch.setattr(api, "CRTM", FakeCRTM)
    ci = []
    assert api.CRTM_IsInitialized(ci)
    assert api.CRTM_Init(["mwsynth_c22"], ci, coeff_dir) == api.SUCCESS
    assert api.CRTM_IsInitialized(ci)
    h = ci[0].handle
    h.close()
    assert not api.CRTM_IsInitialized(ci)
    assert api.CRTM_Destroy(ci) == api.SUCCESS and ci == []
