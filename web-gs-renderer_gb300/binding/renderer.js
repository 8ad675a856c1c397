// renderer.js -- drop-in for src/renderer/renderer.js backed by libwebgs.so through the N-API addon.
// Same public methods (constructor, uploadGsData, setGs, execute); the WebGPU device, canvas and blit
// are replaced by a headless rgba8 image (this.image) the size of a canvas-like {width, height} object,
// which is read every frame as the reference reads its canvas (renderer.js #resize): changing its
// width or height resizes the camera and the image and forces the next frame.
import {createRequire} from "module";
import {Camera} from "../src/renderer/camera.js";  // the reference camera, unchanged (binding folder placed at native/ in that tree)

const require = createRequire(import.meta.url);
const {Native} = require("./build/Release/webgs.node");

export class Renderer {
    #native; #camera; #onProfile; #canvas; #width; #height; #lastTime; #previousGs; #currentGs; #isResized = true;
    #names = new Set();

    // device/context/format of the WebGPU constructor become a canvas-like {width, height}
    constructor(canvas, _context, _format, onProfile) {
        this.#native = new Native({profile: !!onProfile});
        this.#onProfile = onProfile;
        this.#canvas = canvas;
        this.#width = canvas.width;
        this.#height = canvas.height;
        this.#camera = new Camera(this.#width, this.#height);
        this.image = new Uint8Array(this.#width * this.#height * 4);
    }

    uploadGsData(data, name) {
        this.#native.uploadGsData(data, name);
        this.#names.add(name);
    }

    setGs(name) {
        this.#native.setGs(name);  // throws on an unknown name, like fail()
        this.#currentGs = name;
    }

    execute() {
        const now = performance.now();
        const dt = this.#lastTime === undefined ? 0 : (now - this.#lastTime) / 1000;
        this.#lastTime = now;
        this.#resize();
        this.#camera.update(dt);
        if (!this.#names.has(this.#currentGs)) return;
        if (!this.#camera.pollDirty() && !this.#isResized && this.#currentGs === this.#previousGs) return;
        this.#previousGs = this.#currentGs;
        this.#isResized = false;
        const {view, projView, eye, focal, tanFov} = this.#camera.getUniform();
        const block = new ArrayBuffer(176);  // renderer.js:773-797 layout
        const f = new Float32Array(block), u = new Uint32Array(block);
        f.set(view, 0); f.set(projView, 16); f.set(eye, 32); u[35] = 0;
        f.set(focal, 36); f.set(tanFov, 38); f.set([this.#width, this.#height], 40);
        this.#native.render(block, this.image);
        this.#onProfile?.(this.#native.timings());
    }

    // renderer.js #resize: a new canvas size resizes the camera and the output image
    #resize() {
        const {width, height} = this.#canvas;
        if (width === this.#width && height === this.#height) return;
        this.#width = width;
        this.#height = height;
        this.#camera.resize(width, height);
        this.image = new Uint8Array(width * height * 4);
        this.#isResized = true;
    }
}
