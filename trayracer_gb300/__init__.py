"""GB300-native wavefront path tracer: the ray generation -> extend -> shade ->
connect -> accumulate hot path of rdbruijne/trayracer, rebuilt as hand-written
sm_103a CUDA kernels behind a C ABI (include/trayracer.h, libtrayracer.so)."""
from ._abi import (  # noqa: F401
    TR_CLOSURE_DIFFUSE,
    TR_CLOSURE_DISNEY,
    TR_CLOSURE_LAMBERT,
    TR_FLAG_REFERENCE_SAMPLING,
    TR_FLAG_WRITE_AOVS,
    TR_MAX_DEPTH,
    load_library,
)
from .renderer import (BatchRenderer, DeviceRenderer, KernelSettings, RayPickResult, RenderModes,  # noqa: F401
                       SkySettings, TracerError, camera_to_c, settings_for)
from .scenes import (  # noqa: F401
    CameraSpec,
    Scene,
    cornell_box,
    displaced_spheres,
    heightfield,
    instanced_cornell,
    outdoor_heightfield,
    perturbed_materials,
    sphere_batch,
    sphere_scene,
    textured_cornell,
)
from .scenefile import SceneFile, load_scene_file, write_model_cache, write_texture_cache  # noqa: F401,E402
