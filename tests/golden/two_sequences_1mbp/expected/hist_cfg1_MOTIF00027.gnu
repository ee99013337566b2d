set output "hist_cfg1_MOTIF00027.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-34.3554:10.8939]
set yrange [0:114334]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00027.dat" using 1:2 title 'MOTIF00027 (cfg1)' with boxes
