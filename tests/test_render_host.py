"""Host side of the headless volume render (photon_gb300.render) and the
oracle's restatement of the viewer's volume shader, without a GPU."""
import math

import numpy as np

from oracle import oraclepy
from photon_gb300 import casegen, render


def small_case():
    return casegen.tiny_room(12, 10, 9, 0.2, 60e3)


def test_camera_projects_target_to_image_centre():
    c = small_case()
    eye, target = (-3.0, -4.0, 5.0), (1.2, 1.0, 0.9)
    p = render.camera(c, eye, target, width=160, height=90)
    inv = np.array(list(p.inv_vp), np.float64).reshape(4, 4).T      # column-major
    vp = np.linalg.inv(inv)
    clip = vp @ np.array([*target, 1.0])
    ndc = clip[:3] / clip[3]
    assert abs(ndc[0]) < 1e-5 and abs(ndc[1]) < 1e-5 and -1 < ndc[2] < 1
    assert math.isclose(p.step, 0.3 * c.dx, rel_tol=1e-6)
    assert math.isclose(sum(v * v for v in p.sun_dir), 1.0, rel_tol=1e-6)


def test_empty_volume_shows_the_background():
    """No smoke, no fire, nothing hot: transmittance 1 and no light, so every
    pixel is the background colour (src/render/renderer.cpp:281)."""
    c = small_case()
    vol = np.zeros((c.N, 4), np.float32)
    vol[:, 2] = 293.15
    p = render.camera(c, (-3.0, -4.0, 5.0), (1.2, 1.0, 0.9), width=48, height=32, background=(0.2, 0.4, 0.6))
    img = oraclepy.vol_render(c, vol, p)
    np.testing.assert_allclose(img, np.broadcast_to(np.float32([0.2, 0.4, 0.6]), img.shape), atol=1e-7)


def test_more_soot_darkens():
    c = small_case()
    p = render.camera(c, (-3.0, -4.0, 5.0), (1.2, 1.0, 0.9), width=48, height=32, fire=False)
    vol = np.zeros((c.N, 4), np.float32)
    vol[:, 2] = 293.15
    means = []
    for soot in (1e-5, 1e-4, 1e-3):
        vol[:, 0] = soot
        means.append(float(oraclepy.vol_render(c, vol, p).mean()))
    assert means[0] > means[1] > means[2]


def test_fire_lights_spacing_and_power():
    c = small_case()
    hrr = np.zeros(c.N)
    rng = np.random.default_rng(4)
    hot = rng.choice(c.N, 40, replace=False)
    hrr[hot] = rng.uniform(2e5, 2e6, hot.size)
    lights = render.fire_lights(c, hrr, time=0.0)
    assert 1 <= len(lights) <= 8
    pts = np.array([l[:3] for l in lights])
    for a in range(len(pts)):
        for b in range(a + 1, len(pts)):
            assert np.linalg.norm(pts[a] - pts[b]) >= 1.6
    # intensity clamp(sqrt(kW) 0.16, 0, 5) times a flicker of at most 1
    assert all(0 < l[3] <= 5.0 for l in lights)
    # the strongest burning cell carries the first light
    i = int(np.argmax(hrr))
    centre = np.array([c.ox + (i % c.nx + 0.5) * c.dx, c.oy + ((i // c.nx) % c.ny + 0.5) * c.dx,
                       c.oz + (i // (c.nx * c.ny) + 0.5) * c.dx])
    np.testing.assert_allclose(pts[0], centre)


def test_write_ppm(tmp_path):
    img = np.zeros((3, 4, 3), np.float32)
    img[0, 0] = (1.0, 0.0, 0.0)          # bottom-left pixel, rows from the bottom
    path = tmp_path / "x.ppm"
    render.write_ppm(str(path), img)
    data = path.read_bytes()
    header, pixels = data[:11], data[11:]
    assert header == b"P6\n4 3\n255\n"
    px = np.frombuffer(pixels, np.uint8).reshape(3, 4, 3)
    assert tuple(px[2, 0]) == (255, 0, 0)   # last file row is the bottom row
