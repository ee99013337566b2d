set output "hist_cfg1_MOTIF00025.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-82.2118:20.9675]
set yrange [0:160903]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00025.dat" using 1:2 title 'MOTIF00025 (cfg1)' with boxes
