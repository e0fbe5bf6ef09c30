// Prints the byte layout of the reference's kernel parameter structs
// (cpp/src/Renderer/CUDABasedRasterizationInput.h:39-106 and
// CUDABasedRasterizationGradInput.h:26-89) as JSON.  Built only where the
// reference sources are present; refcore.cu checks its replicas against it.
#include <cstddef>
#include <cstdio>

#include "CUDABasedRasterizationInput.h"
#include "CUDABasedRasterizationGradInput.h"

#define F(S, m) std::printf("    \"%s\": %zu,\n", #m, offsetof(S, m))

int main() {
    std::printf("{\n  \"fwd\": {\n");
    using I = CUDABasedRasterizationInput;
    F(I, numberOfCameras); F(I, w); F(I, h); F(I, F); F(I, N); F(I, d_facesVertex); F(I, d_vertexFaces);
    F(I, d_vertexFacesId); F(I, d_textureCoordinates); F(I, d_textureMapIds); F(I, computeNormal); F(I, d_BBoxes);
    F(I, d_projectedVertices); F(I, d_faceNormal); F(I, albedoMode); F(I, shadingMode); F(I, d_inverseExtrinsics);
    F(I, d_inverseProjection); F(I, d_vertices); F(I, d_vertexColor); F(I, texWidth); F(I, texHeight);
    F(I, d_textureMap); F(I, d_shCoeff); F(I, d_cameraExtrinsics); F(I, d_cameraIntrinsics); F(I, d_faceIDBuffer);
    F(I, d_depthBuffer); F(I, d_barycentricCoordinatesBuffer); F(I, d_renderBuffer); F(I, d_vertexNormal);
    F(I, d_normalMap);
    std::printf("    \"sizeof\": %zu\n  },\n  \"bwd\": {\n", sizeof(I));
    using G = CUDABasedRasterizationGradInput;
    F(G, numberOfCameras); F(G, w); F(G, h); F(G, F); F(G, N); F(G, d_facesVertex); F(G, d_textureCoordinates);
    F(G, d_vertexFaces); F(G, d_vertexFacesId); F(G, albedoMode); F(G, shadingMode); F(G, d_inverseExtrinsics);
    F(G, d_inverseProjection); F(G, imageFilterSize); F(G, textureFilterSize); F(G, d_renderBufferGrad);
    F(G, d_targetBufferGrad); F(G, d_vertices); F(G, d_vertexColor); F(G, d_textureMap); F(G, d_shCoeff);
    F(G, d_vertexNormal); F(G, d_barycentricCoordinatesBuffer); F(G, d_faceIDBuffer); F(G, d_targetImage);
    F(G, texWidth); F(G, texHeight); F(G, d_cameraExtrinsics); F(G, d_cameraIntrinsics); F(G, d_vertexPosGrad);
    F(G, d_vertexColorGrad); F(G, d_textureGrad); F(G, d_shCoeffGrad);
    std::printf("    \"sizeof\": %zu\n  }\n}\n", sizeof(G));
    return 0;
}
