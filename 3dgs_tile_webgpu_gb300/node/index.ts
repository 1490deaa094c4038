/**
 * TypeScript face of the gs3d Node-API addon (gs3d_node.c): the surface of the
 * reference's TiledGaussianPipeline (src/renderer/pipeline/TiledGaussianPipeline.ts:65-425)
 * as GaussianPass drives it (src/renderer/GaussianPass.ts:710-805), with the
 * pass running on a GB300 through the gs3d C ABI instead of WebGPU.
 *
 * The Store, LOD selection and streaming protocol are unchanged: they keep
 * producing the packed buffers (GaussianData.ts:10-33,108-138) and hand them
 * to GaussianScene, whose device copy pipelines lease. Render targets are
 * owned by each pipeline (an rgba16f colour buffer and an optional float32
 * depth buffer on the device); readImage() brings the colour back to the
 * host, getResources() exposes the device addresses for CUDA interop.
 *
 * Nothing here blocks the JS thread: render() enqueues the pass, readStats()
 * and readImage() resolve when the GPU has passed their copies.
 */
import { createRequire } from "node:module";

const require = createRequire(import.meta.url);
// Built by `node-gyp rebuild` from binding.gyp.
const addon = require("./build/Release/gs3d_node.node");

export type DepthSortMode = "float32" | "packed16";
export type AntialiasMode = "compensated" | "classic";
export type GaussianBoundaryPolicy = "clip" | "repeat-x" | "repeat-y";
/** "fp32" is the reference's arithmetic; "exact" is bit-identical to the CPU
 * restatement; "half2" evaluates weights in packed half with FP32 blending. */
export type RasterForm = "fp32" | "exact" | "half2";

/** The packed storage buffers of a GaussianData (compact geometry + rgb8e8 SH). */
export interface PackedGaussianData {
  count: number;
  activeCount: number;
  shDegree: number;
  means: Float32Array; // count x 4: xyz, objectId or -1
  scalesOpacity: Uint32Array; // count x 2: f16 ln-scales, f16 opacity
  rotations: Uint32Array; // count: oct101012
  shCoefficients: Uint32Array; // count x (deg+1)^2 rgb8e8, then the active-slot tail
}

/** Constructor options, named as GaussianPass names them (GaussianPass.ts:170-256). */
export interface PipelineOptions {
  depthSortMode?: DepthSortMode;
  antialiasMode?: AntialiasMode;
  intersectionCapacity?: number;
  background?: readonly [number, number, number, number];
  maxRasterizedSplatsPerTile?: number | null;
  rasterChunkSize?: number | null;
  subpixelSampleCulling?: boolean;
  rasterTransmittanceThreshold?: number;
  depthAlphaThreshold?: number;
  filterVariance?: number;
  boundaryPolicy?: GaussianBoundaryPolicy;
  rasterStats?: boolean;
  rasterForm?: RasterForm;
  device?: number;
}

/** What FrameUniforms reads from the camera each frame (FrameUniforms.ts:41-58). */
export interface CameraState {
  projectionMatrix: { elements: ArrayLike<number> };
  matrixWorldInverse: { elements: ArrayLike<number> };
  near: number;
  far: number;
}

/** readStats() (types.ts:94-103) plus the 16-byte output state. */
export interface PassStats {
  visibleGaussianCount: number;
  intersectionCount: number;
  requestedIntersections: number;
  intersectionCapacity: number;
  overflow: boolean;
  rasterWork: { checked: number; blended: number; pixels: number; alphaStopped: number };
  /** attempt, version, demand, overflow (intersections.ts:114-133). */
  outputState: [number, number, number, number];
}

/** getResources(): device addresses of the pass buffers and targets. */
export interface DeviceResources {
  projectedMean: bigint;
  projectedConic: bigint;
  projectedColor: bigint;
  tileCounts: bigint;
  visibleOffsets: bigint;
  depthSortedKeys: bigint;
  depthSortedIds: bigint;
  intersectionOffsets: bigint;
  sortedTileIds: bigint;
  sortedGaussianIds: bigint;
  tileOffsets: bigint;
  outputState: bigint;
  color: bigint;
  depth: bigint;
  tilesX: number;
  tilesY: number;
  intersectionCapacity: number;
}

/** Which store buffer a streamed patch writes (GaussianData attribute order). */
export const enum SceneField {
  Means = 0,
  ScalesOpacity = 1,
  Rotations = 2,
  ShCoefficients = 3,
}

/** A device copy of a store's packed buffers. */
export class GaussianScene {
  readonly handle: object;

  constructor(data: PackedGaussianData) {
    this.handle = addon.createScene(data);
  }

  /** Write a streamed patch at a byte offset of one buffer (the active-slot
   * tail lives at the end of shCoefficients); optionally change activeCount. */
  update(field: SceneField, byteOffset: number, bytes: ArrayBufferView, activeCount?: number): void {
    if (activeCount === undefined) addon.updateScene(this.handle, field, byteOffset, bytes);
    else addon.updateScene(this.handle, field, byteOffset, bytes, activeCount);
  }
}

export class TiledGaussianPipeline {
  private readonly native: {
    updateData(scene: object): void;
    resizeIntersections(capacity: number): void;
    prepareFrame(width: number, height: number, outputDepth: boolean): void;
    setCamera(projection: Float32Array, view: Float32Array, near: number, far: number, objects: Float32Array): void;
    render(attempt: number, resetValid: boolean): void;
    readStats(): Promise<PassStats>;
    readImage(): Promise<ArrayBuffer>;
    getResources(): DeviceResources;
    dispose(): void;
  };
  private readonly projection = new Float32Array(16);
  private readonly view = new Float32Array(16);
  private prepared = false;

  /**
   * @param objectTable the ObjectFrameState rows of the store's objects for
   * the current camera, 40 floats per object (ObjectFrameState.ts:97-119),
   * read once per prepareFrame like the reference's objects.update().
   */
  constructor(
    private data: GaussianScene,
    private readonly camera: CameraState,
    private readonly objectTable: () => Float32Array,
    options: PipelineOptions = {},
  ) {
    const native: Record<string, unknown> = { ...options };
    if (options.maxRasterizedSplatsPerTile === null) native.maxRasterizedSplatsPerTile = 0;
    if (options.rasterChunkSize === null) native.rasterChunkSize = 0;
    this.native = new addon.Pipeline(data.handle, native);
  }

  /** updateData(data) (TiledGaussianPipeline.ts:203-218). */
  updateData(data: GaussianScene): void {
    this.native.updateData(data.handle);
    this.data = data;
  }

  /** resizeIntersections(capacity) (TiledGaussianPipeline.ts:220-231). */
  resizeIntersections(capacity: number): void {
    this.native.resizeIntersections(capacity);
  }

  /** prepareFrame(width, height) (TiledGaussianPipeline.ts:286-322): sizes the
   * targets and reads the camera and object rows for this frame. Throws
   * RangeError when a tile axis exceeds 65,535. */
  prepareFrame(width: number, height: number, outputDepth = false): void {
    this.native.prepareFrame(width, height, outputDepth);
    this.projection.set(Array.from(this.camera.projectionMatrix.elements));
    this.view.set(Array.from(this.camera.matrixWorldInverse.elements));
    this.native.setCamera(this.projection, this.view, this.camera.near, this.camera.far, this.objectTable());
    this.prepared = true;
  }

  /** render(attempt, resetValid) (TiledGaussianPipeline.ts:324-341): enqueues
   * the pass and returns. */
  render(attempt = 1, resetValid = false): void {
    if (!this.prepared) throw new Error("TiledGaussianPipeline must be prepared before rendering");
    this.native.render(attempt, resetValid);
  }

  /** Counters and output state of the last render; one read-back in flight. */
  readStats(): Promise<PassStats> {
    return this.native.readStats();
  }

  /** The 16-byte output state GaussianPass polls (GaussianPass.ts:1019-1079). */
  async readOutputState(): Promise<Uint32Array> {
    const stats = await this.native.readStats();
    return Uint32Array.from(stats.outputState);
  }

  /** The rgba16f colour target of the last render. */
  readImage(): Promise<ArrayBuffer> {
    return this.native.readImage();
  }

  /** getResources() (TiledGaussianPipeline.ts:391-406). */
  getResources(): DeviceResources {
    return this.native.getResources();
  }

  /** dispose() (TiledGaussianPipeline.ts:408-425): releases the scene lease. */
  dispose(): void {
    this.native.dispose();
    this.prepared = false;
  }
}

/** IntersectionCapacityPolicy.next(current, demand) (IntersectionCapacityPolicy.ts:90-100). */
export function capacityNext(
  maximum: number,
  growth: number,
  headroom: number,
  current: number,
  demand: number,
): number | null {
  return addon.capacityNext(maximum, growth, headroom, current, demand);
}
