"""The C++ drop-in layer without a GPU.  libsm2d_ref.so exports the entry
points of the reference's transport path under the names the reference's
callers link against (gpu_transport_wrapper.hpp:21-92,
k1k6_pipeline.cuh:296-416); where SM2D_REFERENCE names the SM_2D tree, the
layer compiled against that tree's own headers defines the same symbols and
every type it exchanges has the same size and member offsets as in
include/sm2d_ref_types.hpp (sm_2d_gb300/shim/check_reference_abi.sh)."""
import ctypes
import os
import subprocess

import pytest

from sm_2d_gb300 import build as B

ENTRY_POINTS = [
    "_ZN5sm_2d15init_device_lutERK4RLUTRNS_16DeviceLUTWrapperE",
    "_ZN5sm_2d16DeviceLUTWrapperC1Ev",
    "_ZN5sm_2d16DeviceLUTWrapperD1Ev",
    "_ZN5sm_2d16get_audit_reportERKNS_17K1K6PipelineStateEii",
    "_ZN5sm_2d17K1K6PipelineState7cleanupEv",
    "_ZN5sm_2d17K1K6PipelineState8allocateEii",
    "_ZN5sm_2d18run_k1_active_maskERK10DevicePsiCPhPKhiiiif",
    "_ZN5sm_2d19init_pipeline_stateERKNS_18K1K6PipelineConfigERK10EnergyGridRK11AngularGridRNS_17K1K6PipelineStateE",
    "_ZN5sm_2d19run_k6_swap_buffersERP10DevicePsiCS2_",
    "_ZN5sm_2d20reset_pipeline_stateERNS_17K1K6PipelineStateEii",
    "_ZN5sm_2d21get_gpu_name_internalB5cxx11Ev",
    "_ZN5sm_2d21run_k3_fine_transportERK10DevicePsiCRS0_PKjiRK10DeviceRLUTRKNS_18K1K6PipelineConfigERNS_17K1K6"
    "PipelineStateE",
    "_ZN5sm_2d22run_k4_bucket_transferER10DevicePsiCPK19DeviceOutflowBucketPKiiiPKfii",
    "_ZN5sm_2d23run_k2_coarse_transportERK10DevicePsiCRS0_PKhPKjiRK10DeviceRLUTRKNS_18K1K6PipelineConfigERNS_17"
    "K1K6PipelineStateE",
    "_ZN5sm_2d25run_k5_conservation_auditERK10DevicePsiCS2_PKdS4_S4_S4_S4_S4_S4_S4_PKfS6_S6_S6_S6_S6_ffddfdiS6_ii"
    "P11AuditReportii",
    "_ZN5sm_2d27run_k1k6_pipeline_transportEP10DevicePsiCS1_RK10DeviceRLUTRK10EnergyGridRK11AngularGridRKNS_18K1K6"
    "PipelineConfigERNS_17K1K6PipelineStateE",
    "_ZN5sm_2d27run_k1k6_pipeline_transportEffffffffijiiffffiiRK11AngularGridRK10EnergyGridRK10DeviceRLUTRKNS_15"
    "TransportConfigERSt6vectorISC_IdSaIdEESaISE_EE",
]


def test_the_layer_exports_the_reference_entry_points():
    B.build()
    lib = ctypes.CDLL(os.path.join(B.OUT, "libsm2d_ref.so"))
    for name in ENTRY_POINTS:
        assert hasattr(lib, name), name
    host = ctypes.CDLL(os.path.join(B.OUT, "libsm2d_ref_host.so"))
    assert hasattr(host, "_Z12GenerateRLUTRK10EnergyGrid")


@pytest.mark.skipif(not os.environ.get("SM2D_REFERENCE"), reason="SM2D_REFERENCE does not name the SM_2D tree")
def test_the_layer_matches_the_reference_headers():
    r = subprocess.run(["sh", os.path.join(B.SHIM, "check_reference_abi.sh")], capture_output=True, text=True)
    assert r.returncode == 0 and "abi ok" in r.stdout, r.stdout + r.stderr
